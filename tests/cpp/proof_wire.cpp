// proof_wire.cpp -- p3g_proof.hpp against the reference's own PCS prover and
// verifier (CPU only; built against the reference's unmodified headers).
//
// TwoAdicFriPcs<BB, BB4, Radix2Dit, flat Poseidon2 MMCS, ExtensionMmcs> commits
// three matrices and opens them at one point with the FRI tests' transcript
// (DuplexChallenger<BabyBear, Poseidon2-16, 16, 8> behind the wrapper of
// fri_test.cpp:100-120) and query proof of work of 8 bits.  Then:
//   1. the proof and the opened values survive encode -> decode -> encode
//      byte for byte;
//   2. the reference's verify accepts the decoded proof and opened values;
//   3. verify rejects the decoded proof after one opened value changes;
//   4. decoding rejects truncated input, a wrong header and a non-canonical
//      field element.
// Prints one line per check; exits non-zero on any failure.

#include "baby_bear.hpp"
#include "extension_field.hpp"
#include "dense_matrix.hpp"
#include "radix2_dit.hpp"
#include "poseidon2_cuda.hpp"
#include "padding_free_sponge.hpp"
#include "truncated_permutation.hpp"
#include "fri_merkle_tree_mmcs.hpp"
#include "fri_extension_mmcs.hpp"
#include "fri_params.hpp"
#include "two_adic_fri_pcs.hpp"
#include "duplex_challenger.hpp"

#include "p3g_proof.hpp"

#include <cstdio>
#include <random>

using namespace p3_field;
using BB = BabyBear;
using Pos = poseidon2::Poseidon2Cuda<BB, 16, 8, 13, 7>;

static Pos make_pos() {
    Pos p;
    std::mt19937 rng(0xdeadbeef);
    for (size_t r = 0; r < 4; ++r)
        for (size_t i = 0; i < 16; ++i) {
            p.initial_external_constants[r][i] = BB(uint32_t(rng() % BB::PRIME));
            p.terminal_external_constants[r][i] = BB(uint32_t(rng() % BB::PRIME));
        }
    for (size_t r = 0; r < 13; ++r) p.internal_constants[r] = BB(uint32_t(rng() % BB::PRIME));
    return p;
}
struct Wrap {
    Pos pos;
    void permute_mut(std::array<BB, 16>& s) const { pos.permute(s.data()); }
};
using Sponge = p3_symmetric::PaddingFreeSponge<Wrap, BB, 16, 8, 8>;
using Trunc = p3_symmetric::TruncatedPermutation<Wrap, BB, 2, 8, 16>;
using Flat = p3_merkle::MerkleTreeMmcs<BB, BB, Sponge, Trunc, 2, 8>;
using EFMmcs = p3_merkle::ExtensionMmcs<BB, BabyBear4, Flat>;
using Pcs = p3_fri::TwoAdicFriPcs<BB, BabyBear4, p3_dft::Radix2Dit<BB>, Flat, EFMmcs>;

struct Transcript {  // the FRI tests' wrapper around DuplexChallenger
    p3_challenger::DuplexChallenger<BB, Wrap, 16, 8> d;
    explicit Transcript(Wrap w) : d(std::move(w)) {}
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

static int report(const char* what, bool ok) {
    std::printf("%s: %s\n", ok ? "ok  " : "FAIL", what);
    return ok ? 0 : 1;
}

int main() {
    int fails = 0;
    const Pos pos = make_pos();
    auto flat = [&] { return Flat(Sponge(Wrap{pos}), Trunc(Wrap{pos})); };
    auto fri = [&] { return p3_fri::FriParameters<EFMmcs>{1, 0, 1, 10, 0, 8, EFMmcs(flat())}; };
    Pcs pcs(p3_dft::Radix2Dit<BB>(), flat(), fri());

    const std::vector<std::pair<size_t, size_t>> shapes = {{6, 5}, {8, 3}, {6, 2}};
    std::vector<std::pair<Pcs::Domain, p3_matrix::RowMajorMatrix<BB>>> ev;
    std::mt19937 rng(42);
    for (const auto& [lh, w] : shapes) {
        std::vector<BB> v((size_t(1) << lh) * w);
        for (auto& x : v) x = BB(uint32_t(rng() % BB::PRIME));
        Pcs::Domain d;
        d.log_n = lh;
        d.shift = BB::one_val();
        ev.push_back({d, p3_matrix::RowMajorMatrix<BB>(std::move(v), w)});
    }
    auto domains = [&] {
        std::vector<Pcs::Domain> ds;
        for (const auto& e : ev) ds.push_back(e.first);
        return ds;
    }();
    auto [commit, pd] = pcs.commit(ev);

    Transcript prover(Wrap{pos});
    prover.observe_commitment(commit);
    const BabyBear4 zeta = prover.sample_challenge<BabyBear4>();
    std::vector<std::vector<BabyBear4>> points(shapes.size(), std::vector<BabyBear4>{zeta});
    auto [opened, proof] = pcs.open({{&pd, points}}, prover);

    // 1. round trip
    const auto pbytes = p3g::wire::encode(proof);
    const auto obytes = p3g::wire::encode(opened);
    const auto proof2 = p3g::wire::decode<Pcs::FullFriProof>(pbytes.data(), pbytes.size());
    const auto opened2 = p3g::wire::decode<Pcs::OpenedValues>(obytes.data(), obytes.size());
    fails += report("proof and opened values: encode -> decode -> encode byte for byte",
                    p3g::wire::encode(proof2) == pbytes && p3g::wire::encode(opened2) == obytes &&
                        opened2 == opened && proof2.final_poly == proof.final_poly &&
                        proof2.query_pow_witness == proof.query_pow_witness);
    std::printf("      proof %zu bytes, opened values %zu bytes\n", pbytes.size(), obytes.size());

    // 2. the reference's verifier on the decoded objects
    auto verify = [&](const Pcs::OpenedValues& ov) {
        Transcript v(Wrap{pos});
        v.observe_commitment(commit);
        const BabyBear4 z = v.sample_challenge<BabyBear4>();
        Pcs::VerifyCommitment vc;
        vc.commitment = commit;
        vc.domains = domains;
        vc.points = std::vector<std::vector<BabyBear4>>(shapes.size(), std::vector<BabyBear4>{z});
        vc.opened_values = ov[0];
        Pcs verifier(p3_dft::Radix2Dit<BB>(), flat(), fri());
        return verifier.verify({vc}, proof2, v);
    };
    fails += report("TwoAdicFriPcs::verify accepts the decoded proof", verify(opened2));

    // 3. a changed opened value is rejected
    auto bad = opened2;
    bad[0][1][0][0].coeffs[0] = bad[0][1][0][0].coeffs[0] + BB(1u);
    fails += report("TwoAdicFriPcs::verify rejects a changed opened value", !verify(bad));

    // 4. malformed input
    bool threw_trunc = false, threw_magic = false, threw_canon = false;
    try {
        (void)p3g::wire::decode<Pcs::FullFriProof>(pbytes.data(), pbytes.size() - 1);
    } catch (const std::invalid_argument&) {
        threw_trunc = true;
    }
    auto wrong = pbytes;
    wrong[0] = 'X';
    try {
        (void)p3g::wire::decode<Pcs::FullFriProof>(wrong.data(), wrong.size());
    } catch (const std::invalid_argument&) {
        threw_magic = true;
    }
    // the first opened value's first coefficient follows the header (8 bytes)
    // and the lengths of the batch, matrix, point and column vectors (4 x 4)
    auto noncanon = obytes;
    const uint32_t first = uint32_t(opened[0][0][0][0].coeffs[0].value());
    bool at_first = std::memcmp(noncanon.data() + 8 + 16, &first, 4) == 0;
    const uint32_t p = BB::PRIME;
    std::memcpy(noncanon.data() + 8 + 16, &p, 4);
    try {
        (void)p3g::wire::decode<Pcs::OpenedValues>(noncanon.data(), noncanon.size());
    } catch (const std::invalid_argument&) {
        threw_canon = true;
    }
    fails += report("decode rejects truncated input, a wrong header and a non-canonical element",
                    threw_trunc && threw_magic && threw_canon && at_first);

    std::printf("%s\n", fails ? "MISMATCH" : "ALL OK");
    return fails ? 1 : 0;
}
