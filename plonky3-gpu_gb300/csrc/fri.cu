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

template <int D, int RF, int RP>
__device__ __noinline__ void chal_duplex(DevChal& c, const P2BB16& p) {
    uint32_t s[16];
    for (int i = 0; i < 16; ++i) s[i] = HBB::absorb(i < int(c.n_in) ? c.in[i] : c.st[i]);
    p2_bb16<D, RF, RP>(s, p);
    for (int i = 0; i < 16; ++i) c.st[i] = HBB::squeeze(s[i]);
    c.n_in = 0;
    for (int i = 0; i < 8; ++i) c.out[i] = c.st[i];
    c.n_out = 8;
}
template <int D, int RF, int RP>
__device__ void chal_absorb(DevChal& c, uint32_t v, const P2BB16& p) {
    c.in[c.n_in++] = v;
    if (c.n_in == 8) chal_duplex<D, RF, RP>(c, p);
}
template <int D, int RF, int RP>
__device__ uint32_t chal_sample(DevChal& c, const P2BB16& p) {
    if (c.n_in > 0 || c.n_out == 0) chal_duplex<D, RF, RP>(c, p);
    return c.out[--c.n_out];
}
__device__ __forceinline__ bb4 bb4_mul_cc(const bb4& a, const bb4& b) { return bb4_mul_cm(a, bb4_to_mont(b)); }

template <int D, int RF, int RP>
__global__ void k_transcript(P2BB16 p, DevChal* dc, ChalStep s) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    DevChal c = *dc;
    if (s.observe_root) {  // observe_merkle_cap with one digest
        c.n_out = 0;
        for (int i = 0; i < 8; ++i) chal_absorb<D, RF, RP>(c, s.observe_root[i], p);
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
            s.final_out[k] = bb4_scale_m(sum, nim);
            wk = bb::mmul(wk, wm);
        }
        for (int k = 0; k < n; ++k) {  // observe_challenge per coefficient
            c.n_out = 0;
            for (int e = 0; e < 4; ++e) chal_absorb<D, RF, RP>(c, s.final_out[k].c[e], p);
        }
        for (int r = 0; r < s.n_arities; ++r) {  // observe_arity: observe(BabyBear(log_arity))
            c.n_out = 0;
            chal_absorb<D, RF, RP>(c, s.arities[r], p);
        }
    }
    if (s.grind_args) {  // the search runs next, from this state
        GrindArgs<uint32_t, 16> a;
        for (int i = 0; i < 16; ++i) a.state[i] = HBB::absorb(i < int(c.n_in) ? c.in[i] : c.st[i]);
        a.n_input = c.n_in;
        a.mask = (uint64_t(1) << s.pow_bits) - 1;
        *s.grind_args = a;
    }
    if (s.take_witness) {  // grind's accepted witness: observe_witness + one sample
        uint64_t w = 0;
        if (s.found) {
            w = *s.found;
            if (w == ~0ull) {
                *s.err = 1;
                w = 0;
            }
        }
        c.n_out = 0;
        chal_absorb<D, RF, RP>(c, uint32_t(w) % bb::P, p);
        chal_absorb<D, RF, RP>(c, uint32_t(w >> 32) % bb::P, p);
        chal_sample<D, RF, RP>(c, p);
        *s.witness_out = w;
    }
    if (s.beta_out) {
        bb4 b;
        for (int e = 0; e < 4; ++e) b.c[e] = chal_sample<D, RF, RP>(c, p);
        *s.beta_out = b;
        for (int k = 0; k < s.log_arity; ++k) b = bb4_mul_cc(b, b);
        *s.beta_pow_out = b;
    }
    for (int q = 0; q < s.num_queries; ++q) {  // sample_bits: one 31-bit sample covers log_max_height
        const uint32_t v = chal_sample<D, RF, RP>(c, p);
        s.query_out[q] = uint64_t(v) & ((uint64_t(1) << s.log_max_height) - 1);
    }
    *dc = c;
}

// Row index of every query in round r's committed matrix: the query index
// shifted right by the log arities of rounds 0..r.
__global__ void k_query_rows(const uint64_t* qidx, int nq, int shift, uint64_t rows, uint64_t* out, uint32_t* err) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    uint64_t r = qidx[q] >> shift;
    if (r >= rows) {  // cannot happen for sampled indices; keep the opening in bounds regardless
        *err = 2;
        r = 0;
    }
    out[q] = r;
}

struct TranscriptFn {
    const P2BB16* p;
    DevChal* c;
    const ChalStep* s;
    cudaStream_t st;
    template <int D, int RF, int RP>
    void operator()() const {
        k_transcript<D, RF, RP><<<1, 1, 0, st>>>(*p, c, *s);
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
    for (int i = 0; i < 8; ++i)
        P3G_REQUIRE(chal->input[i] < bb::P && chal->output[i] < bb::P, "fri: challenger buffers not canonical");
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
    std::vector<size_t> o_rowidx(R), o_rows(R), o_paths(R);
    for (int r = 0; r < R; ++r) {
        const int lrows = rounds[r].log_h - rounds[r].log_arity;
        o_rowidx[r] = take(8 * std::max(nq, 1));
        o_rows[r] = take(4 * size_t(nq) * (4u << rounds[r].log_arity) + 4);
        o_paths[r] = take(4 * size_t(nq) * lrows * 8 + 4);
    }
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
    // ---- query openings of every round's tree
    int shift = 0;
    for (int r = 0; r < R && nq > 0; ++r) {
        shift += rounds[r].log_arity;
        auto* ridx = reinterpret_cast<uint64_t*>(blk + o_rowidx[r]);
        k_query_rows<<<(nq + 127) / 128, 128, 0, st>>>(reinterpret_cast<const uint64_t*>(blk + o_qidx), nq, shift,
                                                       bufs.trees[r]->layer_size[0], ridx, err);
        P3G_LAUNCHED();
        P3G_CUDA(cudaGetLastError());
        open_batch_dev(ctx, bufs.trees[r], ridx, size_t(nq), blk + o_rows[r], blk + o_paths[r], st);
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
