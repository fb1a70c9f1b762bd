// fri.cu -- prove_fri (fri_prover.hpp:35-265) with the data and the
// Fiat-Shamir transcript on the device, so the rounds need no host round trip.
//
// The challenger is the reference's DuplexChallenger<BabyBear, Perm, 16, 8>
// (duplex_challenger.hpp:42-285) kept in device memory and stepped by one
// thread: observations fill the input buffer; a full buffer, or a sample with
// inputs pending or no outputs left, writes the inputs over the first state
// words, permutes (the context's Poseidon2-16) and makes the first 8 words the
// output buffer; samples pop it from the back.
//
// Per round (fri_prover.hpp:83-139): commit current as a (n / arity) x
// (4 arity) BabyBear matrix with the flat MMCS (fri_extension_mmcs.hpp:49-75,
// fri_merkle_tree_mmcs.hpp:55-102); observe the root; proof of work (grind,
// duplex_challenger.hpp:234-251: the parallel search of merkle.cuh reading its
// arguments from the transcript kernel); beta = four samples; fold; add
// beta^arity times the next input where the heights meet.  Then the final
// polynomial (truncate, bit-reverse, inverse DFT, :141-179), its observation
// and the arities' (:181-189), the query proof of work and the query indices
// (:195-210), and every round's opening of every query (:211-257): the
// committed row holding the query's position and the row's Merkle path.
#include <algorithm>
#include <cstring>
#include <vector>

#include "merkle.cuh"

namespace p3g {

struct DevChal {  // same layout as p3g_challenger
    uint32_t st[16];
    uint32_t in[8];
    uint32_t out[8];
    uint32_t n_in, n_out;
};
static_assert(sizeof(DevChal) == sizeof(p3g_challenger), "challenger layout");

constexpr int FRI_MAX_ROUNDS = 32;

// What one transcript launch does, in this order (each step optional).
struct ChalStep {
    const uint32_t* observe_root;     // observe_commitment: 8 words
    // final polynomial: current (2^log_cur BabyBear^4) truncated to 2^log_fpl,
    // bit-reversed, inverse DFT -> final_out; then observe it and the arities
    const bb4* final_cur;
    bb4* final_out;
    int log_fpl;
    uint32_t omega_inv;               // canonical, omega_{2^log_fpl}^-1
    uint32_t n_inv;                   // canonical, 2^-log_fpl
    int n_arities;
    uint8_t arities[FRI_MAX_ROUNDS];
    GrindArgs<uint32_t, 16>* grind_args;  // write the search's arguments (pow_bits > 0) and stop
    uint32_t pow_bits;
    int take_witness;                 // observe the witness (found, or 0) and consume one sample
    const unsigned long long* found;  // the search's result, or null for witness 0
    uint64_t* witness_out;
    bb4* beta_out;                    // sample_challenge
    bb4* beta_pow_out;                // beta^(2^log_arity)
    int log_arity;
    uint64_t* query_out;              // sample_bits(log_max_height) per query
    int num_queries;
    int log_max_height;
    uint32_t* err;                    // set when a search found no witness
};

__device__ __forceinline__ bb4 bb4_mul_cc(const bb4& a, const bb4& b) { return bb4_mul_cm(a, bb4_to_mont(b)); }

// The challenger's steps, run by one warp on a shared-memory copy of its
// state: every lane follows the same (uniform) control flow, lane 0 keeps the
// books, lanes 0-15 hold one state word each through the permutation
// (p2_bb16_coop).  __syncwarp orders the shared-memory updates.
template <int D, int RF, int RP>
__device__ __noinline__ void chal_duplex(DevChal& c, const P2BB16& p, const CoopConsts& cc) {
    const int lane = threadIdx.x, i = lane & 15;
    uint32_t x = HBB::absorb(i < int(c.n_in) ? c.in[i] : c.st[i]);
    x = p2_bb16_coop<D, RF, RP>(x, p, cc, i);
    __syncwarp();
    if (lane < 16) c.st[i] = HBB::squeeze(x);
    __syncwarp();
    if (lane < 8) c.out[lane] = c.st[lane];
    if (lane == 0) {
        c.n_in = 0;
        c.n_out = 8;
    }
    __syncwarp();
}
template <int D, int RF, int RP>
__device__ void chal_absorb(DevChal& c, uint32_t v, const P2BB16& p, const CoopConsts& cc) {
    if (threadIdx.x == 0) c.in[c.n_in++] = v;
    __syncwarp();
    if (c.n_in == 8) chal_duplex<D, RF, RP>(c, p, cc);
}
template <int D, int RF, int RP>
__device__ uint32_t chal_sample(DevChal& c, const P2BB16& p, const CoopConsts& cc) {
    if (c.n_in > 0 || c.n_out == 0) chal_duplex<D, RF, RP>(c, p, cc);
    const uint32_t v = c.out[c.n_out - 1];
    __syncwarp();
    if (threadIdx.x == 0) --c.n_out;
    __syncwarp();
    return v;
}
__device__ __forceinline__ void chal_clear_outputs(DevChal& c) {
    if (threadIdx.x == 0) c.n_out = 0;
    __syncwarp();
}

template <int D, int RF, int RP>
__global__ void __launch_bounds__(32) k_transcript(P2BB16 pp, DevChal* dc, ChalStep s) {
    __shared__ P2BB16 p;  // round constants for the out-of-line permutation
    __shared__ DevChal c;
    const int lane = threadIdx.x;
    for (int k = lane; k < int(sizeof(P2BB16) / 4); k += 32)
        reinterpret_cast<uint32_t*>(&p)[k] = reinterpret_cast<const uint32_t*>(&pp)[k];
    for (int k = lane; k < int(sizeof(DevChal) / 4); k += 32)
        reinterpret_cast<uint32_t*>(&c)[k] = reinterpret_cast<const uint32_t*>(dc)[k];
    __syncwarp();
    const CoopConsts cc = coop_consts(p, lane & 15);
    if (s.observe_root) {  // observe_merkle_cap with one digest
        chal_clear_outputs(c);
        for (int k = 0; k < 8; ++k) chal_absorb<D, RF, RP>(c, s.observe_root[k], p, cc);
    }
    if (s.final_cur) {
        const int n = 1 << s.log_fpl;
        const uint32_t wm = bb::mmul(s.omega_inv, bb::R2), nim = bb::mmul(s.n_inv, bb::R2);
        uint32_t wk = bb::R1;  // omega^-k, Montgomery
        for (int k = 0; k < n; ++k) {
            bb4 sum = {{0, 0, 0, 0}};
            uint32_t wkj = bb::R1;  // omega^-kj
            for (int j = 0; j < n; ++j) {
                const int jr = s.log_fpl ? int(__brev(unsigned(j)) >> (32 - s.log_fpl)) : 0;
                sum = bb4_add(sum, bb4_scale_m(s.final_cur[jr], wkj));
                wkj = bb::mmul(wkj, wk);
            }
            const bb4 coef = bb4_scale_m(sum, nim);
            if (lane == 0) s.final_out[k] = coef;
            chal_clear_outputs(c);  // observe_challenge
            for (int e = 0; e < 4; ++e) chal_absorb<D, RF, RP>(c, coef.c[e], p, cc);
            wk = bb::mmul(wk, wm);
        }
        for (int r = 0; r < s.n_arities; ++r) {  // observe_arity: observe(BabyBear(log_arity))
            chal_clear_outputs(c);
            chal_absorb<D, RF, RP>(c, s.arities[r], p, cc);
        }
    }
    if (s.grind_args && lane < 16) {  // the search runs next, from this state
        const int i = lane;
        s.grind_args->state[i] = HBB::absorb(i < int(c.n_in) ? c.in[i] : c.st[i]);
        if (i == 0) {
            s.grind_args->n_input = c.n_in;
            s.grind_args->mask = (uint64_t(1) << s.pow_bits) - 1;
        }
    }
    if (s.take_witness) {  // grind's accepted witness: observe_witness + one sample
        uint64_t w = 0;
        if (s.found) {
            w = *s.found;
            if (w == ~0ull) {
                if (lane == 0) *s.err = 1;
                w = 0;
            }
        }
        chal_clear_outputs(c);
        chal_absorb<D, RF, RP>(c, uint32_t(w) % bb::P, p, cc);
        chal_absorb<D, RF, RP>(c, uint32_t(w >> 32) % bb::P, p, cc);
        chal_sample<D, RF, RP>(c, p, cc);
        if (lane == 0) *s.witness_out = w;
    }
    if (s.beta_out) {
        bb4 b;
        for (int e = 0; e < 4; ++e) b.c[e] = chal_sample<D, RF, RP>(c, p, cc);
        if (lane == 0) *s.beta_out = b;
        for (int k = 0; k < s.log_arity; ++k) b = bb4_mul_cc(b, b);
        if (lane == 0) *s.beta_pow_out = b;
    }
    for (int q = 0; q < s.num_queries; ++q) {  // sample_bits: one 31-bit sample covers log_max_height
        const uint32_t v = chal_sample<D, RF, RP>(c, p, cc);
        if (lane == 0) s.query_out[q] = uint64_t(v) & ((uint64_t(1) << s.log_max_height) - 1);
    }
    __syncwarp();
    for (int k = lane; k < int(sizeof(DevChal) / 4); k += 32)
        reinterpret_cast<uint32_t*>(dc)[k] = reinterpret_cast<const uint32_t*>(&c)[k];
}

// Every round's opening of every query (fri_prover.hpp:211-257), one block
// per (query, round): the committed row holding the query -- its index is the
// query index shifted right by the log arities of rounds 0..r -- and the
// row's Merkle path (flat tree: a missing sibling is the zero digest).
constexpr int FRI_MAX_DEPTH = 28;
struct FriOpenRound {
    const uint32_t* mat;      // the committed matrix, rows x width
    const uint32_t* digests;  // its tree's layers
    uint32_t* rows_out;       // nq x width
    uint32_t* path_out;       // nq x depth x 8
    uint64_t rows;
    uint32_t width, depth, shift, pad;
    uint64_t layer_off[FRI_MAX_DEPTH];  // in digests
    uint64_t layer_size[FRI_MAX_DEPTH];
};

__global__ void k_fri_open(const FriOpenRound* rounds, const uint64_t* qidx, uint32_t* err) {
    const int q = blockIdx.x;
    const FriOpenRound& rd = rounds[blockIdx.y];
    uint64_t row = qidx[q] >> rd.shift;
    if (row >= rd.rows) {  // cannot happen for sampled indices; stay in bounds regardless
        if (threadIdx.x == 0) *err = 2;
        row = 0;
    }
    for (uint32_t c = threadIdx.x; c < rd.width; c += blockDim.x)
        rd.rows_out[uint64_t(q) * rd.width + c] = rd.mat[row * rd.width + c];
    for (uint32_t e = threadIdx.x; e < rd.depth * 8; e += blockDim.x) {
        const uint32_t l = e / 8, i = e % 8;
        const uint64_t sib = (row >> l) ^ 1;
        rd.path_out[(uint64_t(q) * rd.depth + l) * 8 + i] =
            sib < rd.layer_size[l] ? rd.digests[(rd.layer_off[l] + sib) * 8 + i] : 0u;
    }
}

struct TranscriptFn {
    const P2BB16* p;
    DevChal* c;
    const ChalStep* s;
    cudaStream_t st;
    template <int D, int RF, int RP>
    void operator()() const {
        k_transcript<D, RF, RP><<<1, 32, 0, st>>>(*p, c, *s);
        P3G_LAUNCHED();
        P3G_CUDA(cudaGetLastError());
    }
};

static ChalStep blank_step() {
    ChalStep s;
    std::memset(&s, 0, sizeof s);
    return s;
}

// compute_log_arity_for_round (fri_params.hpp:36-57) over the inputs' heights.
struct FriRound {
    int log_h, log_arity;
    bool mix;  // the next input is added after this round's fold
};
static std::vector<FriRound> plan_rounds(const uint32_t* log_heights, uint32_t n_inputs, const p3g_fri_params& prm) {
    const int log_final = int(prm.log_blowup + prm.log_final_poly_len);
    std::vector<FriRound> rounds;
    int cur = int(log_heights[0]);
    uint32_t idx = 1;
    while (cur > log_final) {
        const bool has_next = idx < n_inputs;
        const int target = has_next ? int(log_heights[idx]) : log_final;
        const int la = cur <= target ? 0 : std::min(cur - target, int(prm.max_log_arity));
        if (la == 0) break;
        FriRound r{cur, la, false};
        cur -= la;
        if (has_next && int(log_heights[idx]) == cur) {
            r.mix = true;
            ++idx;
        }
        rounds.push_back(r);
    }
    return rounds;
}

static void check_fri_args(const uint32_t* log_heights, uint32_t n_inputs, const p3g_fri_params& prm) {
    P3G_REQUIRE(n_inputs >= 1 && n_inputs <= 32, "fri: 1 to 32 inputs");
    for (uint32_t i = 0; i < n_inputs; ++i) {
        P3G_REQUIRE(log_heights[i] <= 27, "fri: input height above 2^27");
        P3G_REQUIRE(i == 0 || log_heights[i] < log_heights[i - 1], "fri: inputs must be sorted by strictly decreasing height");
    }
    P3G_REQUIRE(prm.max_log_arity >= 1, "fri: max_log_arity must be at least 1");
    if (prm.max_log_arity > 3) throw Error(P3G_EUNSUPPORTED, "fri: max_log_arity above 3 (fold arities 2, 4, 8)");
    P3G_REQUIRE(log_heights[n_inputs - 1] > prm.log_blowup + prm.log_final_poly_len,
                "fri: smallest input must be larger than the final domain (fri_prover.hpp:56-67)");
    P3G_REQUIRE(prm.log_final_poly_len <= 10, "fri: log_final_poly_len above 10");
    P3G_REQUIRE(prm.num_queries <= 1024, "fri: more than 1024 queries");
    P3G_REQUIRE(prm.commit_proof_of_work_bits <= 24 && prm.query_proof_of_work_bits <= 24,
                "fri: proof-of-work bits above 24");
}

void fri_rounds(const uint32_t* log_heights, uint32_t n_inputs, const p3g_fri_params& prm, uint32_t* n_rounds,
                uint32_t* log_arities) {
    check_fri_args(log_heights, n_inputs, prm);
    const auto rounds = plan_rounds(log_heights, n_inputs, prm);
    *n_rounds = uint32_t(rounds.size());
    if (log_arities)
        for (size_t r = 0; r < rounds.size(); ++r) log_arities[r] = uint32_t(rounds[r].log_arity);
}

void fri_prove(p3g_ctx* ctx, const void* const* d_inputs, const uint32_t* log_heights, uint32_t n_inputs,
               const p3g_fri_params& prm, p3g_challenger* chal, uint32_t* h_commits, uint64_t* h_commit_witnesses,
               uint32_t* h_final_poly, uint64_t* h_query_witness, uint64_t* h_query_indices, uint32_t* h_rows,
               uint32_t* h_paths, cudaStream_t st) {
    check_fri_args(log_heights, n_inputs, prm);
    for (uint32_t i = 0; i < n_inputs; ++i) P3G_REQUIRE(d_inputs[i], "fri: null input");
    P3G_REQUIRE(chal->n_input < 8 && chal->n_output <= 8, "fri: challenger buffers out of range");
    for (int i = 0; i < 16; ++i) P3G_REQUIRE(chal->sponge_state[i] < bb::P, "fri: challenger state not canonical");
    for (uint32_t i = 0; i < chal->n_input; ++i) P3G_REQUIRE(chal->input[i] < bb::P, "fri: challenger input not canonical");
    for (uint32_t i = 0; i < chal->n_output; ++i)
        P3G_REQUIRE(chal->output[i] < bb::P, "fri: challenger output not canonical");
    if (!ctx->has_p2bb) throw Error(P3G_ESTATE, "Poseidon2 constants for BabyBear are not set");
    const auto rounds = plan_rounds(log_heights, n_inputs, prm);
    const int R = int(rounds.size());
    const int nq = int(prm.num_queries);
    const int log_fpl = int(prm.log_final_poly_len), fpl = 1 << log_fpl;

    // ---- device scratch: one block, downloaded at the end
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
    const size_t o_chal = take(sizeof(DevChal));
    const size_t o_found = take(8 * (R + 1));
    const size_t o_args = take(sizeof(GrindArgs<uint32_t, 16>) * (R + 1));
    const size_t o_beta = take(16 * std::max(R, 1)), o_bpow = take(16 * std::max(R, 1));
    const size_t o_wit = take(8 * (R + 1));
    const size_t o_final = take(16 * fpl);
    const size_t o_qidx = take(8 * std::max(nq, 1));
    const size_t o_err = take(8);
    const size_t o_roots = take(32 * std::max(R, 1));
    std::vector<size_t> o_rows(R), o_paths(R);
    for (int r = 0; r < R; ++r) {
        const int lrows = rounds[r].log_h - rounds[r].log_arity;
        o_rows[r] = take(4 * size_t(nq) * (4u << rounds[r].log_arity) + 4);
        o_paths[r] = take(4 * size_t(nq) * lrows * 8 + 4);
    }
    const size_t o_open = take(sizeof(FriOpenRound) * std::max(R, 1));
    const size_t out_bytes = off;
    struct Bufs {  // everything allocated here, released in stream order on every exit
        p3g_ctx* ctx;
        cudaStream_t st;
        std::vector<void*> v;
        std::vector<p3g_tree*> trees;
        ~Bufs() {
            for (p3g_tree* t : trees) {
                tree_release(ctx, t, st);
                delete t;
            }
            for (void* p : v) ctx->release(p, st);
        }
    } bufs{ctx, st, {}, {}};
    char* blk = static_cast<char*>(ctx->alloc(out_bytes, st));
    bufs.v.push_back(blk);
    auto* dchal = reinterpret_cast<DevChal*>(blk + o_chal);
    auto* found = reinterpret_cast<unsigned long long*>(blk + o_found);
    auto* err = reinterpret_cast<uint32_t*>(blk + o_err);
    P3G_CUDA(cudaMemsetAsync(blk, 0, out_bytes, st));
    P3G_CUDA(cudaMemsetAsync(found, 0xFF, 8 * (R + 1), st));
    DevChal hc;
    std::memcpy(&hc, chal, sizeof hc);
    P3G_CUDA(cudaMemcpyAsync(dchal, &hc, sizeof hc, cudaMemcpyHostToDevice, st));  // pageable: staged now

    // ---- every round's current vector and flat tree, prepared up front
    std::vector<const uint32_t*> cur(R + 1);
    cur[0] = static_cast<const uint32_t*>(d_inputs[0]);
    for (int r = 0; r < R; ++r) {
        const uint64_t n_next = (uint64_t(1) << rounds[r].log_h) >> rounds[r].log_arity;
        void* nb = ctx->alloc(16 * n_next, st);
        bufs.v.push_back(nb);
        cur[r + 1] = static_cast<const uint32_t*>(nb);
        auto* t = new p3g_tree();
        bufs.trees.push_back(t);
        t->field = P3G_BABYBEAR;
        t->mats.push_back(p3g_matrix{cur[r], n_next, 4u << rounds[r].log_arity, 0});
        tree_prepare(ctx, t, 0, true, st, false);
    }

    // the openings' table, uploaded with the rest before any launch
    std::vector<FriOpenRound> open_tab(R);
    for (int r = 0; r < R; ++r) {
        const p3g_tree* t = bufs.trees[r];
        FriOpenRound& o = open_tab[r];
        std::memset(&o, 0, sizeof o);
        o.mat = cur[r];
        o.digests = static_cast<const uint32_t*>(t->d_digests);
        o.rows_out = reinterpret_cast<uint32_t*>(blk + o_rows[r]);
        o.path_out = reinterpret_cast<uint32_t*>(blk + o_paths[r]);
        o.rows = t->layer_size[0];
        o.width = 4u << rounds[r].log_arity;
        o.depth = uint32_t(t->layer_size.size() - 1);
        P3G_REQUIRE(o.depth <= uint32_t(FRI_MAX_DEPTH), "fri: tree too deep");
        int shift = 0;
        for (int k = 0; k <= r; ++k) shift += rounds[k].log_arity;
        o.shift = uint32_t(shift);
        for (uint32_t l = 0; l < o.depth; ++l) {
            o.layer_off[l] = t->layer_off[l];
            o.layer_size[l] = t->layer_size[l];
        }
    }
    if (R) P3G_CUDA(cudaMemcpyAsync(blk + o_open, open_tab.data(), sizeof(FriOpenRound) * R, cudaMemcpyHostToDevice, st));

    auto transcript = [&](const ChalStep& s) { dispatch_bb(ctx, TranscriptFn{&ctx->p2bb, dchal, &s, st}); };
    auto search = [&](int slot, uint32_t bits) {  // one bounded launch: a miss has probability e^-64
        grind_bb_dev(ctx, blk + o_args + sizeof(GrindArgs<uint32_t, 16>) * slot, uint64_t(1) << (bits + 6),
                     found + slot, st);
    };
    // ---- commit phase
    uint32_t next_input = 1;
    for (int r = 0; r < R; ++r) {
        const FriRound& rd = rounds[r];
        p3g_tree* t = bufs.trees[r];
        tree_enqueue(ctx, t, st);
        const uint32_t* root = static_cast<const uint32_t*>(t->d_digests) + t->layer_off.back() * 8;
        P3G_CUDA(cudaMemcpyAsync(blk + o_roots + 32 * r, root, 32, cudaMemcpyDeviceToDevice, st));
        ChalStep s = blank_step();
        s.observe_root = root;
        const uint32_t bits = prm.commit_proof_of_work_bits;
        auto* args = reinterpret_cast<GrindArgs<uint32_t, 16>*>(blk + o_args) + r;
        if (bits > 0) {
            s.grind_args = args;
            s.pow_bits = bits;
            transcript(s);
            search(r, bits);
            s = blank_step();
            s.found = found + r;
        }
        s.take_witness = 1;
        s.witness_out = reinterpret_cast<uint64_t*>(blk + o_wit) + r;
        s.err = err;
        s.beta_out = reinterpret_cast<bb4*>(blk + o_beta) + r;
        s.beta_pow_out = reinterpret_cast<bb4*>(blk + o_bpow) + r;
        s.log_arity = rd.log_arity;
        transcript(s);
        const uint32_t* d_beta = reinterpret_cast<const uint32_t*>(blk + o_beta) + 4 * r;
        fold_bb4(ctx, cur[r], rd.log_h, rd.log_arity, nullptr, const_cast<uint32_t*>(cur[r + 1]), st, d_beta);
        if (rd.mix) {
            const uint64_t n_next = (uint64_t(1) << rd.log_h) >> rd.log_arity;
            bb4_axpy(ctx, const_cast<uint32_t*>(cur[r + 1]), static_cast<const uint32_t*>(d_inputs[next_input]),
                     n_next, nullptr, st, reinterpret_cast<const uint32_t*>(blk + o_bpow) + 4 * r);
            ++next_input;
        }
    }
    // ---- final polynomial, arities, query proof of work, query indices
    {
        ChalStep s = blank_step();
        s.final_cur = reinterpret_cast<const bb4*>(cur[R]);
        s.final_out = reinterpret_cast<bb4*>(blk + o_final);
        s.log_fpl = log_fpl;
        const uint32_t w = bb::two_adic_generator(unsigned(log_fpl));
        s.omega_inv = bb::h_pow(w, uint64_t(fpl) - 1);
        s.n_inv = bb::h_inv(uint32_t(fpl));
        s.n_arities = R;
        for (int r = 0; r < R; ++r) s.arities[r] = uint8_t(rounds[r].log_arity);
        const uint32_t bits = prm.query_proof_of_work_bits;
        if (bits > 0) {
            s.grind_args = reinterpret_cast<GrindArgs<uint32_t, 16>*>(blk + o_args) + R;
            s.pow_bits = bits;
            transcript(s);
            search(R, bits);
            s = blank_step();
            s.found = found + R;
        }
        s.take_witness = 1;
        s.witness_out = reinterpret_cast<uint64_t*>(blk + o_wit) + R;
        s.err = err;
        s.query_out = reinterpret_cast<uint64_t*>(blk + o_qidx);
        s.num_queries = nq;
        int log_max = int(prm.log_blowup + prm.log_final_poly_len);
        for (const auto& rd : rounds) log_max += rd.log_arity;
        s.log_max_height = log_max;
        transcript(s);
    }
    // ---- query openings of every round's tree, one launch
    if (R && nq > 0) {
        k_fri_open<<<dim3(unsigned(nq), unsigned(R)), 64, 0, st>>>(reinterpret_cast<const FriOpenRound*>(blk + o_open),
                                                                 reinterpret_cast<const uint64_t*>(blk + o_qidx), err);
        P3G_LAUNCHED();
        P3G_CUDA(cudaGetLastError());
    }
    // ---- results
    std::vector<char> host(out_bytes);
    P3G_CUDA(cudaMemcpyAsync(host.data(), blk, out_bytes, cudaMemcpyDeviceToHost, st));
    P3G_CUDA(cudaStreamSynchronize(st));
    uint32_t e = 0;
    std::memcpy(&e, host.data() + o_err, 4);
    if (e == 1) throw Error(P3G_ENOTFOUND, "fri: a proof-of-work search found no witness");
    if (e != 0) throw Error(P3G_ECUDA, "fri: query row out of range");
    std::memcpy(chal, host.data() + o_chal, sizeof(DevChal));
    if (h_commits) std::memcpy(h_commits, host.data() + o_roots, 32 * R);
    if (h_commit_witnesses) std::memcpy(h_commit_witnesses, host.data() + o_wit, 8 * R);
    if (h_query_witness) std::memcpy(h_query_witness, host.data() + o_wit + 8 * R, 8);
    if (h_final_poly) std::memcpy(h_final_poly, host.data() + o_final, 16 * fpl);
    if (h_query_indices) std::memcpy(h_query_indices, host.data() + o_qidx, 8 * nq);
    size_t rw = 0, pw = 0;
    for (int r = 0; r < R; ++r) {
        const size_t nr = size_t(nq) * (4u << rounds[r].log_arity);
        const size_t np = size_t(nq) * (rounds[r].log_h - rounds[r].log_arity) * 8;
        if (h_rows) std::memcpy(h_rows + rw, host.data() + o_rows[r], 4 * nr);
        if (h_paths) std::memcpy(h_paths + pw, host.data() + o_paths[r], 4 * np);
        rw += nr;
        pw += np;
    }
}

}  // namespace p3g
