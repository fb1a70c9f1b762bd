// ref_driver.cpp -- runs the reference's own CPU path to produce golden data.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile against the
// reference's unmodified headers (dloghin/plonky3-gpu, src/include) into
// oracle/_ref/ref_driver; tests/golden/make_golden.py runs it and commits the
// resulting fixtures.  The only code of this file's own is argument parsing,
// seeded input generation in the reference tests' convention, a transcript
// adapter over the reference's DuplexChallenger (the member functions that
// TwoAdicFriPcs::open and prove_fri call), and one traits specialisation: the
// reference's Goldilocks has no two-adic generator, so the harness supplies
// omega_{2^k} = 7^((p-1)/2^k) (7 generates F_p^*).
//
// Output: raw little-endian canonical field elements written to <out>.

#include "baby_bear.hpp"
#include "goldilocks.hpp"
#include "extension_field.hpp"
#include "dense_matrix.hpp"
#include "radix2_dit.hpp"
#include "util.hpp"
#include "poseidon2.hpp"
#include "poseidon2_cuda.hpp"
#include "padding_free_sponge.hpp"
#include "truncated_permutation.hpp"
#include "merkle_tree.hpp"
#include "merkle_tree_mmcs.hpp"
#include "merkle_tree_cuda.hpp"
#include "fri_merkle_tree_mmcs.hpp"
#include "fri_extension_mmcs.hpp"
#include "fri_folding.hpp"
#include "fri_params.hpp"
#include "two_adic_fri_pcs.hpp"
#include "duplex_challenger.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

using namespace p3_field;
using p3_matrix::RowMajorMatrix;

namespace p3_dft {
template <>
struct TwoAdicFieldTraits<Goldilocks> {
    static Goldilocks two_adic_generator(size_t bits) {
        return Goldilocks(static_cast<uint64_t>(7)).exp_u64((Goldilocks::PRIME - 1) >> bits);
    }
};
}  // namespace p3_dft

// ---------------------------------------------------------------------------
// Poseidon2 instances, constants drawn in the reference examples' order
// (merkle_tree_cuda_example.cu:53-66; goldilocks_poseidon2_cuda.cu:50-66).
// ---------------------------------------------------------------------------
using BB = BabyBear;
using GL = Goldilocks;
using PosBB = poseidon2::Poseidon2Cuda<BB, 16, 8, 13, 7>;
using PosBBZero = poseidon2::Poseidon2Cuda<BB, 16, 8, 22, 7>;
using PosGL = poseidon2::Poseidon2Cuda<GL, 8, 8, 22, 7>;

static PosBB make_pos_bb() {
    PosBB p;
    std::mt19937 rng(0xdeadbeef);
    for (size_t r = 0; r < 4; ++r)
        for (size_t i = 0; i < 16; ++i) {
            p.initial_external_constants[r][i] = BB(rng() % BB::PRIME);
            p.terminal_external_constants[r][i] = BB(rng() % BB::PRIME);
        }
    for (size_t r = 0; r < 13; ++r) p.internal_constants[r] = BB(rng() % BB::PRIME);
    return p;
}
static PosBBZero make_pos_bb_zero() {
    PosBBZero p;
    for (size_t r = 0; r < 4; ++r)
        for (size_t i = 0; i < 16; ++i) {
            p.initial_external_constants[r][i] = BB();
            p.terminal_external_constants[r][i] = BB();
        }
    for (size_t r = 0; r < 22; ++r) p.internal_constants[r] = BB();
    return p;
}
static PosGL make_pos_gl() {
    PosGL p;
    std::mt19937_64 rng(12345);
    for (size_t r = 0; r < 4; ++r)
        for (size_t i = 0; i < 8; ++i) {
            p.initial_external_constants[r][i] = GL(rng() % GL::PRIME);
            p.terminal_external_constants[r][i] = GL(rng() % GL::PRIME);
        }
    for (size_t r = 0; r < 22; ++r) p.internal_constants[r] = GL(rng() % GL::PRIME);
    return p;
}

template <typename Pos, typename F, size_t W>
struct PermWrap {  // the CPUPermWrapper pattern, merkle_tree_cuda_example.cu:80-91
    Pos pos;
    void permute_mut(std::array<F, W>& s) const { pos.permute(s.data()); }
};
using WrapBB = PermWrap<PosBB, BB, 16>;
using WrapBBZero = PermWrap<PosBBZero, BB, 16>;
using WrapGL = PermWrap<PosGL, GL, 8>;

using SpongeBB = p3_symmetric::PaddingFreeSponge<WrapBB, BB, 16, 8, 8>;
using TruncBB = p3_symmetric::TruncatedPermutation<WrapBB, BB, 2, 8, 16>;
using MmcsBB = p3_merkle_tree::MerkleTreeMmcs<BB, BB, SpongeBB, TruncBB, 8>;
using SpongeBBZ = p3_symmetric::PaddingFreeSponge<WrapBBZero, BB, 16, 8, 8>;
using TruncBBZ = p3_symmetric::TruncatedPermutation<WrapBBZero, BB, 2, 8, 16>;
using MmcsBBZ = p3_merkle_tree::MerkleTreeMmcs<BB, BB, SpongeBBZ, TruncBBZ, 8>;
using SpongeGL = p3_symmetric::PaddingFreeSponge<WrapGL, GL, 8, 4, 4>;
using TruncGL = p3_symmetric::TruncatedPermutation<WrapGL, GL, 2, 4, 8>;
using MmcsGL = p3_merkle_tree::MerkleTreeMmcs<GL, GL, SpongeGL, TruncGL, 4>;
using FlatBB = p3_merkle::MerkleTreeMmcs<BB, BB, SpongeBB, TruncBB, 2, 8>;

// The transcript TwoAdicFriPcs::open and prove_fri drive (fri_prover.hpp,
// two_adic_fri_pcs.hpp:271-510), over the reference's DuplexChallenger with
// the seeded BB16 permutation.
struct OpenTranscript {
    p3_challenger::DuplexChallenger<BB, WrapBB, 16, 8> d;
    explicit OpenTranscript(WrapBB w) : d(std::move(w)) {}
    template <typename C>
    void observe_commitment(const C& c) { d.observe_merkle_cap(c); }
    template <typename EF = BabyBear4>
    EF sample_challenge() { return d.template sample_algebra_element<EF>(); }
    template <typename EF>
    void observe_challenge(const EF& v) { d.template observe_algebra_element<EF>(v); }
    void observe_arity(size_t la) { d.observe(BB(static_cast<uint32_t>(la))); }
    uint64_t grind(size_t bits) { return d.grind(bits); }
    bool check_witness(size_t bits, uint64_t w) { return d.check_witness(bits, w); }
    size_t sample_bits(size_t n) { return d.sample_bits(n); }
};

// ---------------------------------------------------------------------------
// output helpers
// ---------------------------------------------------------------------------
static FILE* g_out = nullptr;
static void put32(uint32_t v) { fwrite(&v, 4, 1, g_out); }
static void put64(uint64_t v) { fwrite(&v, 8, 1, g_out); }
static void put(const BB& v) { put32(v.value()); }
static void put(const GL& v) { put64(v.as_canonical_u64()); }

template <typename F>
static RowMajorMatrix<F> rand_matrix(size_t h, size_t w, uint64_t seed);
template <>
RowMajorMatrix<BB> rand_matrix<BB>(size_t h, size_t w, uint64_t seed) {
    std::mt19937 rng(static_cast<uint32_t>(seed));  // test_ntt_cuda.cpp:55-62 convention
    std::vector<BB> v(h * w);
    for (auto& x : v) x = BB(static_cast<uint32_t>(rng() % BB::PRIME));
    return RowMajorMatrix<BB>(std::move(v), w);
}
template <>
RowMajorMatrix<GL> rand_matrix<GL>(size_t h, size_t w, uint64_t seed) {
    std::mt19937_64 rng(seed);
    std::vector<GL> v(h * w);
    for (auto& x : v) x = GL(rng() % GL::PRIME);
    return RowMajorMatrix<GL>(std::move(v), w);
}

template <typename Tree>
static void put_layers(const Tree& tree) {
    put64(tree.digest_layers.size());
    for (const auto& layer : tree.digest_layers) put64(layer.size());
    for (const auto& layer : tree.digest_layers)
        for (const auto& d : layer)
            for (const auto& e : d) put(e);
}

static std::vector<std::pair<size_t, size_t>> parse_shapes(int argc, char** argv, int from) {
    std::vector<std::pair<size_t, size_t>> s;
    for (int i = from; i < argc; ++i) {
        size_t h = 0, w = 0;
        if (sscanf(argv[i], "%zux%zu", &h, &w) != 2) {
            fprintf(stderr, "bad shape %s\n", argv[i]);
            exit(2);
        }
        s.push_back({h, w});
    }
    return s;
}

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: ref_driver <out> <cmd> args...\n");
        return 2;
    }
    g_out = fopen(argv[1], "wb");
    if (!g_out) return 3;
    std::string cmd = argv[2];

    if (cmd == "consts") {
        // Poseidon2 constants (canonical), BB16 then BB16-zero (none) then GL8.
        PosBB b = make_pos_bb();
        for (auto& r : b.initial_external_constants) for (auto& v : r) put(v);
        for (auto& r : b.terminal_external_constants) for (auto& v : r) put(v);
        for (auto& v : b.internal_constants) put(v);
        PosGL g = make_pos_gl();
        for (auto& r : g.initial_external_constants) for (auto& v : r) put(v);
        for (auto& r : g.terminal_external_constants) for (auto& v : r) put(v);
        for (auto& v : g.internal_constants) put(v);
    } else if (cmd == "kat") {
        put(BB::two_adic_generator(27));
        put32(BabyBear4::dth_root().value());
        auto e28 = BabyBear::ext_two_adic_generator(28);
        for (auto& v : e28) put(v);
        for (size_t k = 0; k <= 27; ++k) put(BB::two_adic_generator(k));
        for (size_t k = 0; k <= 32; ++k) put(p3_dft::TwoAdicFieldTraits<GL>::two_adic_generator(k));
    } else if (cmd == "lde") {
        // lde <bb|gl> <log_h> <w> <log_blowup> <seed> <shift> <bitrev 0|1>
        std::string f = argv[3];
        size_t log_h = atoi(argv[4]), w = atoi(argv[5]), lb = atoi(argv[6]);
        uint64_t seed = strtoull(argv[7], 0, 0), shift = strtoull(argv[8], 0, 0);
        int br = atoi(argv[9]);
        if (f == "bb") {
            p3_dft::Radix2Dit<BB> dft;
            auto m = rand_matrix<BB>(size_t(1) << log_h, w, seed);
            auto out = dft.coset_lde_batch(std::move(m), lb, BB(static_cast<uint32_t>(shift)));
            if (br) p3_matrix::reverse_matrix_index_bits(out);
            for (auto& v : out.values) put(v);
        } else {
            p3_dft::Radix2Dit<GL> dft;
            auto m = rand_matrix<GL>(size_t(1) << log_h, w, seed);
            auto out = dft.coset_lde_batch(std::move(m), lb, GL(shift));
            if (br) p3_matrix::reverse_matrix_index_bits(out);
            for (auto& v : out.values) put(v);
        }
    } else if (cmd == "dft") {
        // dft bb <kind: dft|idft|coset_dft|coset_idft> <log_h> <w> <seed> <shift>
        std::string kind = argv[4];
        size_t log_h = atoi(argv[5]), w = atoi(argv[6]);
        uint64_t seed = strtoull(argv[7], 0, 0), shift = strtoull(argv[8], 0, 0);
        p3_dft::Radix2Dit<BB> dft;
        auto m = rand_matrix<BB>(size_t(1) << log_h, w, seed);
        RowMajorMatrix<BB> out;
        BB s(static_cast<uint32_t>(shift));
        if (kind == "dft") out = dft.dft_batch(std::move(m));
        else if (kind == "idft") out = dft.idft_batch(std::move(m));
        else if (kind == "coset_dft") out = dft.coset_dft_batch(std::move(m), s);
        else out = dft.coset_idft_batch(std::move(m), s);
        for (auto& v : out.values) put(v);
    } else if (cmd == "perm") {
        // perm <bb16|bb16zero|bb16zero_generic|gl8> <n> <seed>
        std::string kind = argv[3];
        size_t n = atoi(argv[4]);
        uint64_t seed = strtoull(argv[5], 0, 0);
        if (kind == "gl8") {
            PosGL p = make_pos_gl();
            std::mt19937_64 rng(seed);
            for (size_t k = 0; k < n; ++k) {
                GL s[8];
                for (auto& x : s) x = GL(rng() % GL::PRIME);
                for (auto& x : s) put(x);
                p.permute(s);
                for (auto& x : s) put(x);
            }
        } else {
            std::mt19937 rng(static_cast<uint32_t>(seed));
            PosBB pb = make_pos_bb();
            PosBBZero pz = make_pos_bb_zero();
            poseidon2::ExternalLayerConstants<BB, 16> ext(
                std::vector<std::array<BB, 16>>(4, std::array<BB, 16>{}),
                std::vector<std::array<BB, 16>>(4, std::array<BB, 16>{}));
            auto generic = poseidon2::create_poseidon2<BB, BB, 16, 7>(ext, std::vector<BB>(22, BB()));
            for (size_t k = 0; k < n; ++k) {
                std::array<BB, 16> s;
                for (auto& x : s) x = BB(static_cast<uint32_t>(rng() % BB::PRIME));
                for (auto& x : s) put(x);
                if (kind == "bb16") pb.permute(s.data());
                else if (kind == "bb16zero") pz.permute(s.data());
                else generic->permute_mut(s);  // fri_test.cpp:57-71 all-zero factory
                for (auto& x : s) put(x);
            }
        }
    } else if (cmd == "hash") {
        // hash <bb16|gl8> <len> <seed> : PaddingFreeSponge::hash_iter
        std::string kind = argv[3];
        size_t len = atoi(argv[4]);
        uint64_t seed = strtoull(argv[5], 0, 0);
        if (kind == "gl8") {
            auto m = rand_matrix<GL>(1, len, seed);
            SpongeGL sp(WrapGL{make_pos_gl()});
            auto d = sp.hash_iter(m.values);
            for (auto& x : d) put(x);
        } else {
            auto m = rand_matrix<BB>(1, len, seed);
            SpongeBB sp(WrapBB{make_pos_bb()});
            auto d = sp.hash_iter(m.values);
            for (auto& x : d) put(x);
        }
    } else if (cmd == "compress") {
        // compress <bb16|gl8> <seed>
        std::string kind = argv[3];
        uint64_t seed = strtoull(argv[4], 0, 0);
        if (kind == "gl8") {
            auto m = rand_matrix<GL>(2, 4, seed);
            TruncGL tr(WrapGL{make_pos_gl()});
            std::array<std::array<GL, 4>, 2> in;
            for (int i = 0; i < 8; ++i) in[i / 4][i % 4] = m.values[i];
            auto d = tr.compress(in);
            for (auto& x : d) put(x);
        } else {
            auto m = rand_matrix<BB>(2, 8, seed);
            TruncBB tr(WrapBB{make_pos_bb()});
            std::array<std::array<BB, 8>, 2> in;
            for (int i = 0; i < 16; ++i) in[i / 8][i % 8] = m.values[i];
            auto d = tr.compress(in);
            for (auto& x : d) put(x);
        }
    } else if (cmd == "mmcs") {
        // mmcs <bb16|bb16zero|gl8> <cap_height> <seed> <h>x<w> ...
        // matrix i is drawn with seed + i.  Also cross-checks the reference's
        // build_merkle_tree_cuda host fallback (BB16) against the MMCS tree.
        std::string kind = argv[3];
        size_t cap = atoi(argv[4]);
        uint64_t seed = strtoull(argv[5], 0, 0);
        auto shapes = parse_shapes(argc, argv, 6);
        if (kind == "gl8") {
            std::vector<RowMajorMatrix<GL>> mats;
            for (size_t i = 0; i < shapes.size(); ++i)
                mats.push_back(rand_matrix<GL>(shapes[i].first, shapes[i].second, seed + i));
            MmcsGL mmcs(SpongeGL(WrapGL{make_pos_gl()}), TruncGL(WrapGL{make_pos_gl()}), cap);
            auto [c, tree] = mmcs.commit(std::move(mats));
            put_layers(tree);
        } else if (kind == "bb16zero") {
            std::vector<RowMajorMatrix<BB>> mats;
            for (size_t i = 0; i < shapes.size(); ++i)
                mats.push_back(rand_matrix<BB>(shapes[i].first, shapes[i].second, seed + i));
            MmcsBBZ mmcs(SpongeBBZ(WrapBBZero{make_pos_bb_zero()}),
                         TruncBBZ(WrapBBZero{make_pos_bb_zero()}), cap);
            auto [c, tree] = mmcs.commit(std::move(mats));
            put_layers(tree);
        } else {
            std::vector<RowMajorMatrix<BB>> mats, mats2;
            for (size_t i = 0; i < shapes.size(); ++i) {
                mats.push_back(rand_matrix<BB>(shapes[i].first, shapes[i].second, seed + i));
                mats2.push_back(mats.back());
            }
            MmcsBB mmcs(SpongeBB(WrapBB{make_pos_bb()}), TruncBB(WrapBB{make_pos_bb()}), cap);
            auto [c, tree] = mmcs.commit(std::move(mats));
            auto tree2 = p3_merkle_tree::build_merkle_tree_cuda<BB, 16, 8, 8, 8, 13, 7>(
                std::move(mats2), make_pos_bb(), cap);
            if (tree2.digest_layers != tree.digest_layers) {
                fprintf(stderr, "build_merkle_tree_cuda host path disagrees with MMCS\n");
                return 4;
            }
            put_layers(tree);
        }
    } else if (cmd == "commit_matrix") {
        // commit_matrix <height> <width> <seed> : flat p3_merkle::MerkleTreeMmcs
        size_t h = atoi(argv[3]), w = atoi(argv[4]);
        uint64_t seed = strtoull(argv[5], 0, 0);
        auto m = rand_matrix<BB>(h, w, seed);
        FlatBB mmcs(SpongeBB(WrapBB{make_pos_bb()}), TruncBB(WrapBB{make_pos_bb()}));
        auto [c, pd] = mmcs.commit_matrix(m.values, w);
        put64(pd.tree.size());
        for (auto& l : pd.tree) put64(l.size());
        for (auto& l : pd.tree) for (auto& d : l) for (auto& e : d) put(e);
    } else if (cmd == "commit") {
        // commit <log_h> <w> <log_blowup> <seed> <cap> : LDE (bit-reversed rows) + MMCS
        size_t log_h = atoi(argv[3]), w = atoi(argv[4]), lb = atoi(argv[5]);
        uint64_t seed = strtoull(argv[6], 0, 0);
        size_t cap = atoi(argv[7]);
        p3_dft::Radix2Dit<BB> dft;
        auto lde = dft.coset_lde_batch(rand_matrix<BB>(size_t(1) << log_h, w, seed), lb, BB::generator());
        p3_matrix::reverse_matrix_index_bits(lde);
        std::vector<RowMajorMatrix<BB>> mats;
        mats.push_back(std::move(lde));
        MmcsBB mmcs(SpongeBB(WrapBB{make_pos_bb()}), TruncBB(WrapBB{make_pos_bb()}), cap);
        auto [c, tree] = mmcs.commit(std::move(mats));
        put_layers(tree);
    } else if (cmd == "pcs_open") {
        // pcs_open <seed> <log_h>x<w> ... : TwoAdicFriPcs::commit as in pcs_commit, then
        // open every matrix at one point zeta sampled from the transcript.  Writes zeta,
        // alpha (the first challenge open samples), every opened value, the number of
        // FRI commit-phase rounds, the log arity of round 0 and its commitment (the
        // Merkle root of the bit-reversed reduced-opening vector of the tallest height).
        uint64_t seed = strtoull(argv[3], 0, 0);
        auto shapes = parse_shapes(argc, argv, 4);
        using EFMmcs = p3_merkle::ExtensionMmcs<BB, BabyBear4, FlatBB>;
        using Pcs = p3_fri::TwoAdicFriPcs<BB, BabyBear4, p3_dft::Radix2Dit<BB>, FlatBB, EFMmcs>;
        auto mk = [] { return FlatBB(SpongeBB(WrapBB{make_pos_bb()}), TruncBB(WrapBB{make_pos_bb()})); };
        p3_fri::FriParameters<EFMmcs> fri{1, 0, 1, 10, 0, 8, EFMmcs(mk())};
        Pcs pcs(p3_dft::Radix2Dit<BB>(), mk(), std::move(fri));
        std::vector<std::pair<typename Pcs::Domain, RowMajorMatrix<BB>>> ev;
        size_t max_log = 0;
        for (size_t i = 0; i < shapes.size(); ++i) {
            typename Pcs::Domain d;
            d.log_n = shapes[i].first;
            d.shift = BB::one_val();
            ev.push_back({d, rand_matrix<BB>(size_t(1) << shapes[i].first, shapes[i].second, seed + i)});
            max_log = std::max(max_log, shapes[i].first + 1);
        }
        auto [commit, pd] = pcs.commit(std::move(ev));
        OpenTranscript tr(WrapBB{make_pos_bb()});
        tr.observe_commitment(commit);
        const BabyBear4 zeta = tr.sample_challenge<BabyBear4>();
        OpenTranscript peek = tr;
        const BabyBear4 alpha = peek.sample_challenge<BabyBear4>();
        std::vector<std::vector<BabyBear4>> points(shapes.size(), std::vector<BabyBear4>{zeta});
        std::vector<std::pair<const typename Pcs::PcsProverData*, std::vector<std::vector<BabyBear4>>>> od;
        od.push_back({&pd, points});
        auto [opened, proof] = pcs.open(od, tr);
        for (size_t k = 0; k < 4; ++k) put(zeta[k]);
        for (size_t k = 0; k < 4; ++k) put(alpha[k]);
        for (const auto& mat : opened[0])
            for (const auto& pt : mat)
                for (const auto& v : pt)
                    for (size_t k = 0; k < 4; ++k) put(v[k]);
        put32(uint32_t(proof.commit_phase_commits.size()));
        put32(uint32_t(p3_fri::compute_log_arity_for_round(max_log, false, 0, 1, 1)));
        for (const auto& e : proof.commit_phase_commits.at(0)[0]) put(e);
        // then: the PCS commitment, every commit-phase root and the final polynomial
        for (const auto& e : commit[0]) put(e);
        for (const auto& c : proof.commit_phase_commits)
            for (const auto& e : c[0]) put(e);
        put32(uint32_t(proof.final_poly.size()));
        for (const auto& v : proof.final_poly)
            for (size_t k = 0; k < 4; ++k) put(v[k]);
        // then: the query-phase proof-of-work witness (query_proof_of_work_bits = 8)
        put64(proof.query_pow_witness);
        // then every query's commit-phase openings: per round the sibling values
        // and the Merkle path of the committed row
        put32(uint32_t(proof.query_proofs.size()));
        for (const auto& qp : proof.query_proofs) {
            put32(uint32_t(qp.commit_phase_openings.size()));
            for (const auto& step : qp.commit_phase_openings) {
                put32(uint32_t(step.log_arity));
                put32(uint32_t(step.sibling_values.size()));
                for (const auto& v : step.sibling_values)
                    for (size_t k = 0; k < 4; ++k) put(v[k]);
                put32(uint32_t(step.opening_proof.size()));
                for (const auto& d : step.opening_proof)
                    for (const auto& e : d) put(e);
            }
        }
    } else if (cmd == "grind") {
        // grind <seed> <n_obs> <bits>... : the reference's DuplexChallenger (BB16,
        // rate 8, seeded permutation) observes n_obs seeded values, then for each
        // bits: grind(bits) and one more sample().  (Its grind does not compile
        // for the reference's Goldilocks, which has no FIELD_BITS.)
        uint64_t seed = strtoull(argv[3], 0, 0);
        size_t n_obs = atoi(argv[4]);
        p3_challenger::DuplexChallenger<BB, WrapBB, 16, 8> ch(WrapBB{make_pos_bb()});
        std::mt19937 rng(static_cast<uint32_t>(seed));
        for (size_t i = 0; i < n_obs; ++i) ch.observe(BB(static_cast<uint32_t>(rng() % BB::PRIME)));
        for (int a = 5; a < argc; ++a) {
            put64(ch.grind(atoi(argv[a])));
            put(ch.sample());
        }
    } else if (cmd == "pcs_commit") {
        // pcs_commit <seed> <log_h>x<w> ... : TwoAdicFriPcs::commit (log_blowup 1,
        // domain shift 1 as in fri_test.cpp) with the seeded BB16 Poseidon2.
        uint64_t seed = strtoull(argv[3], 0, 0);
        auto shapes = parse_shapes(argc, argv, 4);
        using EFMmcs = p3_merkle::ExtensionMmcs<BB, BabyBear4, FlatBB>;
        using Pcs = p3_fri::TwoAdicFriPcs<BB, BabyBear4, p3_dft::Radix2Dit<BB>, FlatBB, EFMmcs>;
        auto mk = [] { return FlatBB(SpongeBB(WrapBB{make_pos_bb()}), TruncBB(WrapBB{make_pos_bb()})); };
        p3_fri::FriParameters<EFMmcs> fri{1, 0, 1, 10, 0, 8, EFMmcs(mk())};
        Pcs pcs(p3_dft::Radix2Dit<BB>(), mk(), std::move(fri));
        std::vector<std::pair<typename Pcs::Domain, RowMajorMatrix<BB>>> ev;
        for (size_t i = 0; i < shapes.size(); ++i) {
            typename Pcs::Domain d;
            d.log_n = shapes[i].first;
            d.shift = BB::one_val();
            ev.push_back({d, rand_matrix<BB>(size_t(1) << shapes[i].first, shapes[i].second, seed + i)});
        }
        auto [commit, pd] = pcs.commit(std::move(ev));
        for (auto& d : commit) for (auto& e : d) put(e);
    } else if (cmd == "fold") {
        // fold <log_height> <log_arity> <seed> <beta_mode 0 random | 1 beta = t_0 of row 0>
        size_t log_h = atoi(argv[3]), la = atoi(argv[4]);
        uint64_t seed = strtoull(argv[5], 0, 0);
        int mode = atoi(argv[6]);
        std::mt19937 rng(static_cast<uint32_t>(seed));  // fri_fold_cuda_example.cu:91-100
        auto rnd = [&] { return BB(static_cast<uint32_t>(rng() % BB::PRIME)); };
        std::vector<BabyBear4> v(size_t(1) << log_h);
        for (auto& e : v) e = BabyBear4({rnd(), rnd(), rnd(), rnd()});
        BabyBear4 beta({rnd(), rnd(), rnd(), rnd()});
        if (mode == 1) {
            // row 0: x = omega^0 = 1, t_0 = 1 -> exercise the beta == t_i fast path
            beta = BabyBear4::one_val();
        }
        auto out = p3_fri::TwoAdicFriFolding<BB, BabyBear4>::fold_matrix(log_h, la, beta, v);
        for (int i = 0; i < 4; ++i) put(beta[i]);
        for (auto& e : out) for (int i = 0; i < 4; ++i) put(e[i]);
    } else {
        fprintf(stderr, "unknown cmd %s\n", cmd.c_str());
        return 2;
    }
    fclose(g_out);
    return 0;
}
