/*
 * p3g.h -- C ABI of the GB300 trace-commitment library (libp3g_gb300.so).
 *
 * Plain pointers and sizes only.  "d_" pointers are device (HBM) pointers on
 * the context's GPU; "h_" pointers are host memory.  `stream` is a
 * cudaStream_t (NULL = the legacy default stream).  Every call is
 * stream-ordered and asynchronous unless it says it returns host data, in
 * which case it synchronises `stream` before returning.
 *
 * Field elements are canonical little-endian integers: BabyBear
 * (p = 2^31 - 2^27 + 1) as uint32, Goldilocks (p = 2^64 - 2^32 + 1) as uint64,
 * BabyBear^4 = BabyBear[x]/(x^4 - 11) as 4 x uint32 (coefficient 0 first).
 * Matrices are row-major (RowMajorMatrix, dense_matrix.hpp:21-293 of the
 * reference).
 *
 * Errors: every function returns a P3G_* status; the message of the last
 * failure on the calling thread is available from p3g_last_error().  There is
 * no CPU fallback: a call either runs on the GPU or fails.
 *
 * Threading: a context is externally synchronised (one host thread at a
 * time); distinct contexts are independent.
 */
#ifndef P3G_H
#define P3G_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define P3G_API __attribute__((visibility("default")))
#else
#define P3G_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define P3G_VERSION 1

enum p3g_status {
    P3G_OK = 0,
    P3G_EINVAL = 1,      /* bad argument (reference: std::invalid_argument) */
    P3G_ENOMEM = 2,      /* device allocation failed */
    P3G_ECUDA = 3,       /* CUDA runtime error (reference: P3_CUDA_CHECK runtime_error) */
    P3G_ETIMEOUT = 4,    /* a bounded device or host wait ran out */
    P3G_EUNSUPPORTED = 5,/* shape or parameter outside what this build supports */
    P3G_ESTATE = 6,      /* missing set-up (e.g. no Poseidon2 constants) */
    P3G_ENOTFOUND = 7    /* a bounded search ended without a result (p3g_grind) */
};

enum p3g_field {
    P3G_BABYBEAR = 0,
    P3G_GOLDILOCKS = 1
};

typedef struct p3g_ctx p3g_ctx;
typedef struct p3g_tree p3g_tree;

/* ------------------------------------------------------------ basics */
P3G_API int p3g_version(void);
P3G_API const char *p3g_status_string(int status);
/* Copies the calling thread's last error message (NUL-terminated). */
P3G_API int p3g_last_error(char *buf, size_t len);
/* Number of CUDA kernels this library has launched in the process so far
 * (instrumentation for benchmarks and tests). */
P3G_API uint64_t p3g_kernel_launches(void);

/* Creates a context on `device`: root-of-unity tables, a stream-ordered
 * device memory pool.  Replaces the per-call set-up of NttCuda
 * (ntt_cuda.hpp:272-289) and build_merkle_tree_cuda (merkle_tree_cuda.hpp:360). */
P3G_API int p3g_ctx_create(int device, p3g_ctx **out);
P3G_API int p3g_ctx_destroy(p3g_ctx *ctx);
P3G_API int p3g_stream_synchronize(p3g_ctx *ctx, void *stream);

/* The context's device memory pool: bytes the pool holds from the driver
 * (reserved) and bytes handed out (used), now and at their peaks.  Any output
 * may be NULL. */
P3G_API int p3g_ctx_memory(p3g_ctx *ctx, uint64_t *reserved, uint64_t *used, uint64_t *reserved_high,
                           uint64_t *used_high);

/* Stream-ordered allocations from the context pool (what the library itself
 * uses for scratch and outputs), plus copies, so that callers without a CUDA
 * runtime binding can drive the library. */
P3G_API int p3g_malloc(p3g_ctx *ctx, size_t bytes, void **d_ptr, void *stream);
P3G_API int p3g_free(p3g_ctx *ctx, void *d_ptr, void *stream);
P3G_API int p3g_memcpy_h2d(p3g_ctx *ctx, void *d_dst, const void *h_src, size_t bytes, void *stream);
P3G_API int p3g_memcpy_d2h(p3g_ctx *ctx, void *h_dst, const void *d_src, size_t bytes, void *stream);

/* ------------------------------------------------------------ Poseidon2
 * Sets the permutation used by the MMCS calls of `field`.  Replaces
 * poseidon2::Poseidon2Cuda<F, WIDTH, ROUNDS_F, ROUNDS_P, D> (poseidon2_cuda.hpp:37-117)
 * together with its sponge/compression wrappers:
 *   BabyBear:   width 16, PaddingFreeSponge rate 8, digest 8,
 *               TruncatedPermutation<2, 8, 16> (padding_free_sponge.hpp:63-113,
 *               truncated_permutation.hpp:61-76);
 *   Goldilocks: width 8, rate 4, digest 4, TruncatedPermutation<2, 4, 8>.
 * rounds_f even and <= 8, rounds_p <= 32, sbox_degree in {3, 5, 7}.
 * initial/terminal: [rounds_f/2][width] canonical elements; internal: [rounds_p]. */
P3G_API int p3g_set_poseidon2(p3g_ctx *ctx, int field, uint32_t width, uint32_t rounds_f,
                      uint32_t rounds_p, uint32_t sbox_degree, const void *h_initial,
                      const void *h_terminal, const void *h_internal);

/* Batch permutation of n states (n x width elements, in place on device).
 * Replaces poseidon2_permute_kernel (poseidon2_cuda.hpp:156-166). */
P3G_API int p3g_poseidon2_permute(p3g_ctx *ctx, int field, void *d_states, size_t n, void *stream);

/* ------------------------------------------------------------ DFT / LDE
 * Coset low-degree extension of a batch of columns:
 *   out = coset_lde_batch(in, log_blowup, shift)            (radix2_dit.hpp:221-233)
 *   and, if bitrev_out, reverse_matrix_index_bits(out)      (util.hpp:33-45)
 * in:  (1 << log_h) x width, natural order;  out: (1 << (log_h + log_blowup)) x width.
 * Replaces NttCuda<F>::coset_lde_batch (ntt_cuda.hpp:369-378, 607-649).
 * in and out must not overlap.  Supports log_h <= 26 (P3G_EUNSUPPORTED above);
 * heights above 2^21 take one more pass over the data and scratch of the
 * trace's size per call. */
P3G_API int p3g_coset_lde(p3g_ctx *ctx, int field, const void *d_in, uint32_t log_h, uint32_t width,
                  uint32_t log_blowup, uint64_t shift, int bitrev_out, void *d_out, void *stream);

/* The Dft interface's other members on a batch of columns:
 *   P3G_DFT        Radix2Dit::dft_batch        (radix2_dit.hpp:82-121)
 *   P3G_IDFT       Radix2Dit::idft_batch       (radix2_dit.hpp:136-160)
 *   P3G_COSET_DFT  Radix2Dit::coset_dft_batch  (radix2_dit.hpp:173-186), shift used
 *   P3G_COSET_IDFT Radix2Dit::coset_idft_batch (radix2_dit.hpp:194-210), shift used
 * and, if bitrev_out, reverse_matrix_index_bits of the result.  Replaces
 * NttCuda's dft_batch / idft_batch / coset_dft_batch / coset_idft_batch
 * (ntt_cuda.hpp:310-356).  in, out: (1 << log_h) x width, natural order
 * unless bitrev_out; in and out must not overlap.  Supports log_h <= 26. */
enum p3g_dft_kind {
    P3G_DFT = 0,
    P3G_IDFT = 1,
    P3G_COSET_DFT = 2,
    P3G_COSET_IDFT = 3
};
P3G_API int p3g_dft(p3g_ctx *ctx, int field, int kind, const void *d_in, uint32_t log_h, uint32_t width,
                    uint64_t shift, int bitrev_out, void *d_out, void *stream);

/* BabyBear-only variant of p3g_coset_lde that allocates nothing and needs no
 * context.  It has no counterpart in the reference.  It is for callers that
 * must not enter the CUDA allocator while they prove -- a service that
 * reserves its device memory up front so that no request can fail or
 * fragment the heap on an allocation, or a host whose own memory manager owns
 * the GPU -- whereas p3g_coset_lde takes its scratch from the context's pool.
 * Scratch lives in a fixed 16 MiB device array (plus 96 KiB of root tables)
 * that every GPU loading the library holds until exit; requests needing more
 * scratch are rejected with P3G_EINVAL (with bit-reversed output that is
 * about (1 << log_h) * width <= 4M elements).  The first call on a device
 * sets the arrays up (address lookup, synchronous table copy) with that
 * device current: make it before any stream capture.  All calls share the
 * array, so calls that overlap on the GPU race; serialise them.  Arguments
 * as for p3g_coset_lde: shift canonical (below p) and non-zero, width up to
 * 2^24, log_h up to 21. */
P3G_API int p3g_coset_lde_bb_noalloc(const void *d_in, uint32_t log_h, uint32_t width,
                                     uint32_t log_blowup, uint32_t shift, int bitrev_out,
                                     void *d_out, void *stream);

/* ------------------------------------------------------------ MMCS */
typedef struct {
    const void *d_data;   /* row-major height x width, device */
    uint64_t height;      /* power of two */
    uint32_t width;
    uint32_t reserved;
} p3g_matrix;

/* Mixed-height MerkleTreeMmcs::commit (merkle_tree_mmcs.hpp:100-107,
 * merkle_tree.hpp:84-185): stable sort by height, leaf = sponge over the
 * concatenated rows of the tallest matrices, compress per level, inject
 * shorter matrices, stop at 2^cap_height nodes.  The tree keeps the digest
 * layers on the device and references (does not copy) the matrices, which
 * must stay alive until p3g_tree_free.  h_cap_out (may be NULL) receives the
 * cap, 2^cap_height digests (or fewer if the tree is shorter); the call then
 * synchronises `stream`.  Replaces build_merkle_tree_cuda (merkle_tree_cuda.hpp:360-621). */
P3G_API int p3g_mmcs_commit(p3g_ctx *ctx, int field, const p3g_matrix *mats, size_t n_mats,
                    uint32_t cap_height, p3g_tree **tree_out, void *h_cap_out, void *stream);

/* Flat single-matrix MMCS, p3_merkle::MerkleTreeMmcs::commit_matrix
 * (fri_merkle_tree_mmcs.hpp:55-102): any height >= 1, odd layers padded with
 * a zero digest, commitment = the root.  h_root_out (may be NULL) gets one digest. */
P3G_API int p3g_commit_matrix(p3g_ctx *ctx, int field, const void *d_flat, uint64_t height,
                      uint32_t width, p3g_tree **tree_out, void *h_root_out, void *stream);

/* Layer geometry: number of digest layers and the number of digests in each
 * (layer 0 = leaves; capacity of h_layer_sizes >= 64). */
P3G_API int p3g_tree_info(const p3g_tree *tree, uint32_t *n_layers, uint64_t *h_layer_sizes,
                  uint32_t *digest_elems);
/* Device pointer to digest layer `layer` (digests contiguous, digest_elems each). */
P3G_API int p3g_tree_layer_ptr(const p3g_tree *tree, uint32_t layer, const void **d_ptr);
/* Device pointer of leaf matrix i (in commit order). */
P3G_API int p3g_tree_leaf_ptr(const p3g_tree *tree, uint32_t i, const void **d_ptr);

/* MerkleTreeMmcs::open_batch (merkle_tree_mmcs.hpp:120-152) for n queries:
 * for each query index q, the row index/(max_h/h_i) of every matrix i (rows
 * concatenated in commit order into h_rows, sum(width_i) elements per query)
 * and the sibling path (n_layers-1 digests per query into h_proof).  Synchronises. */
P3G_API int p3g_mmcs_open_batch(p3g_ctx *ctx, const p3g_tree *tree, const uint64_t *h_indices,
                        size_t n_queries, void *h_rows, void *h_proof, void *stream);

/* Releases the tree's device memory (digest layers and owned LDEs) in stream
 * order on `stream`: work already queued on `stream` may still read it. */
P3G_API int p3g_tree_free(p3g_ctx *ctx, p3g_tree *tree, void *stream);

/* ------------------------------------------------------------ commit pipeline */
typedef struct {
    const void *d_trace;  /* (1 << log_h) x width evaluations, device */
    uint32_t log_h;
    uint32_t width;
    uint32_t log_blowup;
    uint32_t reserved;
    uint64_t shift;       /* coset shift, canonical */
} p3g_trace;

/* The trace-commitment hot path: for every trace, the coset LDE with rows in
 * bit-reversed order, then one mixed-height MMCS commit over all LDEs (the
 * LDEs are owned by the returned tree; see p3g_tree_leaf_ptr).  With one
 * trace this is the per-trace commit; with many it is the batched commit, and
 * traces of equal (log_h, log_blowup, shift) run their LDEs as one launch per
 * pass.  Shifts must be canonical and non-zero; log_h up to 26. */
P3G_API int p3g_commit_traces(p3g_ctx *ctx, int field, const p3g_trace *traces, size_t n_traces,
                      uint32_t cap_height, p3g_tree **tree_out, void *h_cap_out, void *stream);

/* p3g_commit_traces with the traces in HOST memory (d_trace is a host
 * pointer; pinned memory gives asynchronous copies).  Each trace is copied in
 * column chunks of 512-byte rows (a trace of 2^14 rows or more given first
 * starts with chunks of 1/4, 1/4 and 1/2 of that) on a second stream; each
 * chunk's LDE starts as soon as its copy has landed, and its row hashes as
 * soon as its LDE is written, resuming the sponge of the chunks before it
 * wherever the row so far is a multiple of the sponge rate long.  So the
 * copies overlap the LDEs and the hashing.  The commitment is the same as for
 * the unsplit traces (a leaf hashes the concatenated rows of equal-height
 * matrices in order, merkle_tree.hpp:84-185); the tree's leaf matrices are
 * the column chunks, in trace order. */
P3G_API int p3g_commit_traces_host(p3g_ctx *ctx, int field, const p3g_trace *traces, size_t n_traces,
                                   uint32_t cap_height, p3g_tree **tree_out, void *h_cap_out, void *stream);

/* ------------------------------------------------------------ batched commit as one graph */
typedef struct p3g_plan p3g_plan;

typedef struct {
    const void *d_in;     /* 2^log_height BabyBear^4 values, device */
    void *d_out;          /* 2^(log_height - log_arity) values, device */
    uint32_t log_height;
    uint32_t log_arity;
    uint32_t beta[4];     /* folding challenge, canonical */
} p3g_fold_job;

/* Plans the batched commit of a fixed batch of traces (shapes and device
 * pointers fixed; contents may change between launches): allocates every
 * LDE, digest layer and work descriptor once and captures the whole step --
 * all LDEs (bit-reversed rows) list-scheduled over n_streams streams, the
 * mixed-height MMCS (merkle_tree_mmcs.hpp:100-107) and, if `fold` is given,
 * one fold_matrix (fri_folding.hpp:200) -- into a CUDA graph.  n_streams = 0
 * lets an autotuner pick the stream count (cached per shape; persisted to the
 * JSON file named by the P3G_TUNE_CACHE environment variable).  The batched
 * counterpart of TwoAdicFriPcs::commit's LDE + commit (two_adic_fri_pcs.hpp:207-266). */
P3G_API int p3g_plan_commit(p3g_ctx *ctx, int field, const p3g_trace *traces, size_t n_traces,
                            uint32_t cap_height, const p3g_fold_job *fold, uint32_t n_streams,
                            p3g_plan **plan_out);
/* p3g_plan_commit with every input in pinned HOST memory: each trace's
 * d_trace and the fold's d_in are page-locked host pointers (cudaMallocHost or
 * cudaHostRegister; P3G_EINVAL otherwise), read on every launch.  The graph
 * copies them into device buffers the plan owns, on a copy stream, in the
 * order the LDE streams take the traces, and each LDE waits only for its own
 * trace, so the copies overlap the LDEs of the traces copied before.  The
 * fold's d_out stays a device pointer.  The end-to-end form of the batched
 * commit: host data in, commitment (p3g_plan_info's tree) out. */
P3G_API int p3g_plan_commit_host(p3g_ctx *ctx, int field, const p3g_trace *traces, size_t n_traces,
                                 uint32_t cap_height, const p3g_fold_job *fold, uint32_t n_streams,
                                 p3g_plan **plan_out);
/* Replays the plan's graph on `stream` (one cudaGraphLaunch). */
P3G_API int p3g_plan_launch(p3g_ctx *ctx, p3g_plan *plan, void *stream);
/* The plan's tree (use with p3g_tree_info/_layer_ptr/_leaf_ptr/p3g_mmcs_open_batch;
 * freed by p3g_plan_destroy, not p3g_tree_free), the stream count in use and
 * the number of kernels one launch runs. */
P3G_API int p3g_plan_info(const p3g_plan *plan, const p3g_tree **tree, uint32_t *n_streams,
                          uint64_t *kernels_per_launch);
P3G_API int p3g_plan_destroy(p3g_ctx *ctx, p3g_plan *plan);

/* ------------------------------------------------------------ serving loop */
typedef struct p3g_server p3g_server;

typedef struct {
    uint64_t id;
    const void *h_trace;  /* (1 << log_h) x width BabyBear, host memory (pinned for
                             asynchronous copies); valid until the result is polled */
    uint32_t log_h;
    uint32_t width;       /* >= 4 */
    uint32_t log_blowup;
    uint32_t reserved;
    uint64_t shift;
    uint32_t beta[4];     /* fold challenge */
} p3g_request;

typedef struct {
    uint64_t id;
    int32_t status;       /* P3G_OK, P3G_ENOMEM (larger than the budget), ... */
    uint32_t reserved;
    uint32_t root[8];     /* MMCS commitment of the bit-reversed LDE */
    uint32_t fold_head[4];/* first value of the fold */
    uint64_t t_submit_ns, t_admit_ns, t_done_ns;  /* steady-clock timestamps */
} p3g_result;

/* A continuous-batching commit+fold service on the context's GPU.  Requests
 * queue in submission order; a worker thread admits the head as soon as one of
 * `max_slots` streams is free and its device-memory footprint fits
 * `mem_budget_bytes` (0 = 80% of the currently free memory), so requests that
 * arrive while others run overlap on the device.  Each request: host->device
 * copy, coset LDE (bit-reversed rows), Poseidon2 MMCS commit, and fold_matrix
 * (log_arity 1) of the LDE's first four columns read as BabyBear^4 values.  The
 * LDE, tree and folded vector stay resident (and count against the budget)
 * until p3g_server_release; p3g_server_open serves MerkleTreeMmcs::open_batch
 * queries on them and p3g_server_read_fold copies the folded vector out.  The reference has no serving layer; this mirrors its
 * commit (merkle_tree_mmcs.hpp:100-107), open_batch (:120-152) and
 * fold_matrix (fri_folding.hpp:200) per request. */
P3G_API int p3g_server_create(p3g_ctx *ctx, uint32_t max_slots, uint64_t mem_budget_bytes,
                              p3g_server **server_out);
P3G_API int p3g_server_submit(p3g_server *server, const p3g_request *request);
/* Moves up to max_results completed results (in completion order) to `out`. */
P3G_API int p3g_server_poll(p3g_server *server, p3g_result *out, size_t max_results, size_t *n_out);
P3G_API int p3g_server_pending(p3g_server *server, uint64_t *queued, uint64_t *in_flight,
                               uint64_t *resident, uint64_t *bytes_used);
P3G_API int p3g_server_open(p3g_server *server, uint64_t id, const uint64_t *h_indices,
                            size_t n_queries, void *h_rows, void *h_proof);
/* The resident fold output of a completed request: n_values = H / 2 BabyBear^4
 * values (4 canonical u32 each, H = 2^(log_h + log_blowup)) into h_out, in
 * fold_matrix's output order.  Synchronous. */
P3G_API int p3g_server_read_fold(p3g_server *server, uint64_t id, void *h_out, uint64_t n_values);
P3G_API int p3g_server_release(p3g_server *server, uint64_t id);
/* Stops the worker; queued requests are dropped, in-flight ones are waited for. */
P3G_API int p3g_server_destroy(p3g_server *server);

/* ------------------------------------------------------------ FRI
 * TwoAdicFriFolding<BabyBear, BabyBear4>::fold_matrix (fri_folding.hpp:200-222)
 * with fold_row's interpolation (fri_folding.hpp:74-189); log_arity in 1..3.
 * d_in: 2^log_height BabyBear4 values; d_out: 2^(log_height - log_arity).
 * Replaces fold_matrix_cuda_device (fri_fold_cuda.hpp:251-277). */
P3G_API int p3g_fold_matrix_bb4(p3g_ctx *ctx, const void *d_in, uint32_t log_height,
                        uint32_t log_arity, const uint32_t h_beta[4], void *d_out,
                        void *stream);

/* y[i] += a * x[i] for n BabyBear^4 values on the device: prove_fri's mix-in of
 * the next reduced opening, current += beta^arity * next (fri_prover.hpp:127-138).
 * With p3g_commit_matrix (the round's commitment of current viewed as
 * (n / arity) x (4 arity) BabyBear, fri_extension_mmcs.hpp:49-75) and
 * p3g_fold_matrix_bb4 this is every device step of the FRI commit phase. */
P3G_API int p3g_bb4_axpy(p3g_ctx *ctx, void *d_y, const void *d_x, uint64_t n, const uint32_t h_a[4],
                         void *stream);

/* ------------------------------------------------------------ proof of work
 * DuplexChallenger::grind (duplex_challenger.hpp:234-251) for the challenger
 * DuplexChallenger<F, Perm, WIDTH, RATE> over the context's Poseidon2
 * permutation: BabyBear WIDTH 16, RATE 8; Goldilocks WIDTH 8, RATE 4.
 * Called by prove_fri for the commit- and query-phase witnesses
 * (fri_prover.hpp:116, 195).
 *
 * The challenger's state: h_sponge_state (WIDTH elements) and its pending
 * inputs h_input (n_input < RATE elements, in observation order); values are
 * u32 (BabyBear, canonical) or u64 (Goldilocks).  The pending outputs do not
 * matter: observing the witness discards them.  Writes the smallest witness w
 * for which observe_witness(w) (elements F(w mod 2^32), F(w >> 32)) followed
 * by sample() gives an element whose canonical value has its low `bits` bits
 * zero -- the witness the reference's sequential search returns.  The caller
 * then applies check_witness(bits, w) to its own challenger, which performs
 * the same observe-and-sample that grind leaves behind.
 * bits must be below FIELD_BITS (31 BabyBear, 64 Goldilocks); max_witness
 * bounds the search (0 = unbounded, as in the reference); P3G_ENOTFOUND if no
 * witness below it passes.  Synchronises the stream. */
P3G_API int p3g_grind(p3g_ctx *ctx, int field, const void *h_sponge_state, const void *h_input,
                      uint32_t n_input, uint32_t bits, uint64_t max_witness, uint64_t *witness_out,
                      void *stream);

/* ------------------------------------------------------------ FRI prover
 * prove_fri (fri_prover.hpp:35-265) for BabyBear / BabyBear^4 over inputs
 * resident on the device, with the Fiat-Shamir transcript on the device as
 * well: the challenger is DuplexChallenger<BabyBear, Perm, 16, 8> over the
 * context's Poseidon2-16, stepped by one device thread, so the rounds run
 * without a host round trip.  The transcript calls are those of the FRI tests'
 * transcript wrapper (fri_test.cpp:100-120): observe_commitment observes the
 * root, sample_challenge draws four samples, observe_challenge observes four
 * coefficients, observe_arity observes BabyBear(log_arity), grind is
 * DuplexChallenger::grind. */
typedef struct {
    uint32_t log_blowup;
    uint32_t log_final_poly_len;     /* <= 10 */
    uint32_t max_log_arity;          /* 1..3 */
    uint32_t num_queries;            /* <= 1024 */
    uint32_t commit_proof_of_work_bits;  /* <= 24 */
    uint32_t query_proof_of_work_bits;   /* <= 24 */
} p3g_fri_params;                    /* FriParameters (fri_params.hpp:9-24) without the MMCS */

/* DuplexChallenger<BabyBear, Perm, 16, 8>'s state (duplex_challenger.hpp:46-49),
 * canonical values; input[0..n_input) and output[0..n_output) are live. */
typedef struct {
    uint32_t sponge_state[16];
    uint32_t input[8];
    uint32_t output[8];
    uint32_t n_input;   /* < 8 */
    uint32_t n_output;  /* <= 8 */
} p3g_challenger;

/* The commit-phase rounds prove_fri makes for these input heights and their
 * log arities (compute_log_arity_for_round, fri_params.hpp:36-57), for sizing
 * p3g_fri_prove's outputs.  log_arities has room for 32. */
P3G_API int p3g_fri_rounds(const uint32_t *log_heights, uint32_t n_inputs, const p3g_fri_params *params,
                           uint32_t *n_rounds, uint32_t *log_arities);

/* d_inputs[i]: 2^log_heights[i] BabyBear^4 values (the reduced openings, rows
 * bit-reversed), heights strictly decreasing, the smallest above
 * log_blowup + log_final_poly_len (fri_prover.hpp:50-67); they are not
 * modified.  challenger: the state before prove_fri on entry, after it on
 * return.  Outputs (host, any may be NULL), for R rounds with log arities a_r
 * on heights 2^h_r:
 *   h_commits           R x 8      each round's root (commit_phase_commits)
 *   h_commit_witnesses  R          (commit_pow_witnesses)
 *   h_final_poly        2^log_final_poly_len x 4
 *   h_query_witness     1          (query_pow_witness)
 *   h_query_indices     num_queries (sample_bits(log_max_height), :207)
 *   h_rows              rounds in order, num_queries x (4 << a_r) each: the
 *                       committed row holding the query (sibling_values = the
 *                       row without the query's position, :221-241)
 *   h_paths             rounds in order, num_queries x (h_r - a_r) x 8 each:
 *                       the row's Merkle path (opening_proof, :243-244)
 * The input MMCS openings at the query indices are the caller's (its own trees,
 * p3g_mmcs_open_batch).  P3G_ENOTFOUND if a proof-of-work search (one bounded
 * launch of 2^(bits+6) candidates) found no witness.  Synchronises the stream. */
P3G_API int p3g_fri_prove(p3g_ctx *ctx, const void *const *d_inputs, const uint32_t *log_heights,
                          uint32_t n_inputs, const p3g_fri_params *params, p3g_challenger *challenger,
                          uint32_t *h_commits, uint64_t *h_commit_witnesses, uint32_t *h_final_poly,
                          uint64_t *h_query_witness, uint64_t *h_query_indices, uint32_t *h_rows,
                          uint32_t *h_paths, void *stream);

/* ------------------------------------------------------------ PCS open
 * TwoAdicFriPcs::open's two passes over a BabyBear LDE resident on the device
 * (two_adic_fri_pcs.hpp:271-410).  d_lde: (1 << log_n) x width evaluations on
 * the coset shift * <omega_n>, rows in natural order or, if bitrev_rows, in
 * bit-reversed order (as p3g_commit_traces leaves them); 1 to 4 BabyBear^4
 * points (h_points: n_points x 4 canonical u32).
 *
 * Opened values, by barycentric interpolation (compute_diff_invs and
 * interpolate_coset_with_precomputation, interpolation.hpp:93-180):
 * h_out[p][c] (n_points x width x 4) = column c's polynomial at point p.
 * Synchronises the stream. */
P3G_API int p3g_pcs_open_values(p3g_ctx *ctx, const void *d_lde, uint32_t log_n, uint32_t width, int bitrev_rows,
                                uint32_t shift, const uint32_t *h_points, uint32_t n_points, uint32_t *h_out,
                                void *stream);
/* The reduced opening of one matrix (two_adic_fri_pcs.hpp:350-410), added in
 * place to d_q ((1 << log_n) x 4 BabyBear^4 on the device):
 *   q[k] += sum_p sum_c alpha^(alpha_pow + p*width + c)
 *                       * (opened[p][c] - lde[k][c]) / (z_p - shift * omega_n^k),
 * k the natural row index; q[k] is stored at k, or at bitrev(k) if q_bitrev
 * (the order prove_fri takes).  h_opened: n_points x width x 4 from
 * p3g_pcs_open_values; n_points * width <= 10240. */
P3G_API int p3g_pcs_reduce(p3g_ctx *ctx, const void *d_lde, uint32_t log_n, uint32_t width, int bitrev_rows,
                           uint32_t shift, const uint32_t *h_points, uint32_t n_points, const uint32_t *h_opened,
                           const uint32_t h_alpha[4], uint64_t alpha_pow, int q_bitrev, void *d_q, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* P3G_H */
