// adapters_standin.cpp -- drives the C++ adapters (p3g_adapters.hpp) with
// minimal stand-ins for the reference's types, on machines without the
// reference's headers.  The stand-ins have exactly the members the adapters
// touch: BabyBear / Goldilocks (value(), as_canonical_u64(), explicit
// construction from the canonical integer), BabyBear4 (operator[]),
// RowMajorMatrix (values, width(), height(), (vector, width) constructor),
// and the MMCS classes' Digest / Commitment / ProverData types.
//
//   adapters_standin lde <bb|gl> <in> <out> <log_h> <width> <added_bits> <shift>
//   adapters_standin commit_matrix <in> <out> <height> <width>
//   adapters_standin mmcs <bb|gl> <in> <out> <cap_height> <h0> <w0> [<h1> <w1> ...]
//   adapters_standin build_tree <bb|gl> <in> <out> <cap_height> <h0> <w0> ...   (build_merkle_tree_cuda)
//   adapters_standin fold <in> <out> <log_height> <log_arity>
//   adapters_standin fold_cuda <in> <out> <log_height> <log_arity>   (host and device forms)
//   adapters_standin dft <bb|gl> <in> <out> <log_h> <width> <kind 0-3> <shift>
//   adapters_standin challenger <out> <seed> <n_obs> <bits>...
//   adapters_standin prove_fri <in> <out> <challenger> <nq> <log_blowup> <log_fpl> <max_la> <cpow> <qpow> <log_h>...
//   adapters_standin pcs_commit <in> <out> <log_blowup> <shift> <log_h0> <w0> [<log_h1> <w1> ...]
//       (TwoAdicFriPcs::commit's composition over GpuDft and GpuInputMmcs;
//        <out> receives the root digest, then the flat committed matrix)
//
// <in> holds canonical little-endian words (u32 BabyBear, u64 Goldilocks;
// for mmcs the matrices back to back; for fold 4 beta coefficients, then
// the values); <out> receives the result (for the trees every digest layer
// from the leaves up).  Poseidon2 is the BabyBear-16 x^7 8+13 permutation
// with constants from std::mt19937(0xdeadbeef) and the Goldilocks-8 x^7 8+22
// one from std::mt19937_64(12345), initial and terminal drawn interleaved.
// The challenger command observes n_obs values std::mt19937(seed)() % p in a
// GpuDuplexChallenger<BabyBear, ..., 16, 8> (host steps permuted through
// p3g_poseidon2_permute), then for each bits grinds and samples once more,
// writing the witness (u64) and the sample (u32).

#include "p3g_adapters.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <random>
#include <string>

namespace standin {

struct BabyBear {
    static constexpr uint32_t PRIME = 0x78000001u;
    uint32_t v = 0;
    BabyBear() = default;
    explicit BabyBear(uint32_t x) : v(x % PRIME) {}
    uint32_t value() const { return v; }
    bool operator==(const BabyBear& o) const { return v == o.v; }
};
struct Goldilocks {
    static constexpr uint64_t PRIME = 0xFFFFFFFF00000001ull;
    uint64_t v = 0;
    Goldilocks() = default;
    explicit Goldilocks(uint64_t x) : v(x) {}
    uint64_t as_canonical_u64() const { return v >= PRIME ? v - PRIME : v; }
    bool operator==(const Goldilocks& o) const { return as_canonical_u64() == o.as_canonical_u64(); }
};
struct BabyBear4 {
    static constexpr size_t DEGREE = 4;
    std::array<BabyBear, 4> coeffs{};
    BabyBear& operator[](size_t i) { return coeffs[i]; }
    const BabyBear& operator[](size_t i) const { return coeffs[i]; }
};

template <class F>
struct RowMajorMatrix {
    std::vector<F> values;
    size_t width_;
    RowMajorMatrix(std::vector<F> v, size_t w) : values(std::move(v)), width_(w) {}
    size_t width() const { return width_; }
    size_t height() const { return width_ ? values.size() / width_ : 0; }
};

struct Radix2Dit {  // only the empty-matrix case reaches the base class
    template <class M, class F>
    M coset_lde_batch(M m, size_t, const F&) {
        return m;
    }
};

template <class F, size_t N>
struct FlatMmcs {
    using Digest = std::array<F, N>;
    using Commitment = std::vector<Digest>;
    struct ProverData {
        std::vector<F> flat_data;
        size_t height = 0, width = 0;
        std::vector<std::vector<Digest>> tree;
    };
};

template <class F, size_t N>
struct MixedMmcs {
    using Digest = std::array<F, N>;
    struct Commitment {
        std::vector<Digest> cap;
        explicit Commitment(std::vector<Digest> c) : cap(std::move(c)) {}
    };
    struct ProverData {
        std::vector<RowMajorMatrix<F>> leaves;
        std::vector<std::vector<Digest>> digest_layers;
    };
    struct Sponge {};
    struct Trunc {};
    MixedMmcs(Sponge, Trunc, size_t) {}
};

template <class F, size_t W, size_t RF, size_t RP, uint64_t D>
struct Poseidon2Cuda {  // the members build_merkle_tree_cuda reads (poseidon2_cuda.hpp:37-45)
    F initial_external_constants[RF / 2][W];
    F terminal_external_constants[RF / 2][W];
    F internal_constants[RP];
};

}  // namespace standin

namespace p3_fri {  // the reference's FRI types (fri_params.hpp, fri_proof.hpp), as the adapter declares them
template <typename FriMmcs>
struct FriParameters {
    size_t log_blowup, log_final_poly_len, max_log_arity, num_queries, commit_proof_of_work_bits,
        query_proof_of_work_bits;
    FriMmcs mmcs;
};
template <typename Challenge, typename FriMmcs>
struct CommitPhaseProofStep {
    uint8_t log_arity = 0;
    std::vector<Challenge> sibling_values;
    typename FriMmcs::OpeningProof opening_proof;
};
template <typename Challenge, typename FriMmcs, typename InputProof>
struct QueryProof {
    InputProof input_proof;
    std::vector<CommitPhaseProofStep<Challenge, FriMmcs>> commit_phase_openings;
};
template <typename Challenge, typename FriMmcs, typename Witness, typename InputProof>
struct FriProof {
    std::vector<typename FriMmcs::Commitment> commit_phase_commits;
    std::vector<Witness> commit_pow_witnesses;
    std::vector<QueryProof<Challenge, FriMmcs, InputProof>> query_proofs;
    std::vector<Challenge> final_poly;
    Witness query_pow_witness{};
};
}  // namespace p3_fri

namespace p3_merkle_tree {  // the reference's tree type, as the adapter's declaration expects
template <typename F, typename W, size_t DIGEST_ELEMS>
struct MerkleTree {
    std::vector<standin::RowMajorMatrix<F>> leaves;
    std::vector<std::vector<std::array<W, DIGEST_ELEMS>>> digest_layers;
};
}  // namespace p3_merkle_tree

using namespace standin;

static std::vector<unsigned char> read_file(const char* path) {
    std::ifstream f(path, std::ios::binary);
    return std::vector<unsigned char>(std::istreambuf_iterator<char>(f), {});
}
static void write_file(const char* path, const std::vector<unsigned char>& b) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(b.data()), std::streamsize(b.size()));
}
template <class F, size_t N>
static void append_layers(std::vector<unsigned char>& out, const std::vector<std::vector<std::array<F, N>>>& l) {
    for (const auto& layer : l)
        for (const auto& d : layer) {
            auto w = p3g::to_words(std::vector<F>(d.begin(), d.end()));
            out.insert(out.end(), w.begin(), w.end());
        }
}

static void set_constants() {
    std::mt19937 r32(0xdeadbeef);
    std::vector<std::array<BabyBear, 16>> bi(4), bt(4);
    for (size_t r = 0; r < 4; ++r)
        for (size_t i = 0; i < 16; ++i) {
            bi[r][i] = BabyBear(uint32_t(r32() % BabyBear::PRIME));
            bt[r][i] = BabyBear(uint32_t(r32() % BabyBear::PRIME));
        }
    std::vector<BabyBear> bin;
    for (size_t r = 0; r < 13; ++r) bin.push_back(BabyBear(uint32_t(r32() % BabyBear::PRIME)));
    p3g::Context::get().set_poseidon2(bi, bt, bin, 7);

    std::mt19937_64 r64(12345);
    std::vector<std::array<Goldilocks, 8>> gi(4), gt(4);
    for (size_t r = 0; r < 4; ++r)
        for (size_t i = 0; i < 8; ++i) {
            gi[r][i] = Goldilocks(r64() % Goldilocks::PRIME);
            gt[r][i] = Goldilocks(r64() % Goldilocks::PRIME);
        }
    std::vector<Goldilocks> gin;
    for (size_t r = 0; r < 22; ++r) gin.push_back(Goldilocks(r64() % Goldilocks::PRIME));
    p3g::Context::get().set_poseidon2(gi, gt, gin, 7);
}

struct DevicePermBB {  // Perm for the challenger's host steps: one state through the GPU permutation
    void permute_mut(std::array<BabyBear, 16>& s) const {
        uint32_t w[16];
        for (size_t i = 0; i < 16; ++i) w[i] = s[i].value();
        p3g::DeviceBuffer d(sizeof w);
        d.upload(w, sizeof w);
        p3g::check(p3g_poseidon2_permute(p3g::Context::get().handle(), P3G_BABYBEAR, d.get(), 1, nullptr));
        d.download(w, sizeof w);
        for (size_t i = 0; i < 16; ++i) s[i] = BabyBear(w[i]);
    }
};

static int run_challenger(int argc, char** a) {
    const uint32_t seed = uint32_t(std::strtoul(a[3], nullptr, 0));
    const size_t n_obs = std::strtoul(a[4], nullptr, 0);
    p3g::GpuDuplexChallenger<BabyBear, DevicePermBB, 16, 8> ch{DevicePermBB{}};
    std::mt19937 rng(seed);
    for (size_t i = 0; i < n_obs; ++i) ch.observe(BabyBear(uint32_t(rng() % BabyBear::PRIME)));
    std::vector<unsigned char> out;
    for (int i = 5; i < argc; ++i) {
        const uint64_t w = ch.grind(std::strtoul(a[i], nullptr, 0));
        const uint32_t v = ch.sample().value();
        out.insert(out.end(), reinterpret_cast<const unsigned char*>(&w), reinterpret_cast<const unsigned char*>(&w) + 8);
        out.insert(out.end(), reinterpret_cast<const unsigned char*>(&v), reinterpret_cast<const unsigned char*>(&v) + 4);
    }
    // state() / set_state() carry the transcript over: a copy continues identically
    ch.observe(BabyBear(5u));
    p3g::GpuDuplexChallenger<BabyBear, DevicePermBB, 16, 8> copy{DevicePermBB{}};
    copy.set_state(ch.state());
    for (int k = 0; k < 10; ++k)
        if (!(copy.sample() == ch.sample())) return 6;
    write_file(a[2], out);
    return 0;
}

// gpu_prove_fri with stand-ins for the FRI MMCS (its Commitment / OpeningProof
// types) and an input MMCS whose opening records the index.
struct FriMmcsStandin {
    using Digest = std::array<BabyBear, 8>;
    using Commitment = std::vector<Digest>;
    using OpeningProof = std::vector<Digest>;
};
struct IndexMmcs {
    struct ProverData {};
    struct OpeningProof {
        size_t row_index = 0;
    };
    void open(size_t index, const std::vector<ProverData>&, OpeningProof& p) const { p.row_index = index; }
};
struct FriTranscript {  // the wrapper shape of fri_test.cpp:100-120
    p3g::GpuDuplexChallenger<BabyBear, DevicePermBB, 16, 8> inner{DevicePermBB{}};
};

// prove_fri <in> <out> <challenger> <num_queries> <log_blowup> <log_final_poly_len> <max_log_arity>
//           <commit_pow_bits> <query_pow_bits> <log_h0> [<log_h1> ...]
static int run_prove_fri(int argc, char** a) {
    auto in = read_file(a[2]);
    auto chb = read_file(a[4]);
    if (chb.size() != sizeof(p3g_challenger)) return 2;
    p3g_challenger st;
    std::memcpy(&st, chb.data(), sizeof st);
    p3_fri::FriParameters<FriMmcsStandin> prm{std::strtoul(a[6], nullptr, 0), std::strtoul(a[7], nullptr, 0),
                                              std::strtoul(a[8], nullptr, 0), std::strtoul(a[5], nullptr, 0),
                                              std::strtoul(a[9], nullptr, 0), std::strtoul(a[10], nullptr, 0),
                                              FriMmcsStandin{}};
    std::vector<std::vector<BabyBear4>> inputs;
    size_t off = 0;
    for (int i = 11; i < argc; ++i) {
        const size_t n = size_t(1) << std::strtoul(a[i], nullptr, 0);
        auto words = p3g::from_words<BabyBear>(in.data() + off, 4 * n);
        std::vector<BabyBear4> v(n);
        for (size_t k = 0; k < n; ++k)
            for (int e = 0; e < 4; ++e) v[k][e] = words[4 * k + e];
        inputs.push_back(std::move(v));
        off += 16 * n;
    }
    FriTranscript tr;
    tr.inner.set_state(st);
    auto proof = p3g::gpu_prove_fri<BabyBear, BabyBear4, FriMmcsStandin, FriTranscript, uint64_t, IndexMmcs,
                                    IndexMmcs::OpeningProof>(prm, std::move(inputs), tr, {}, IndexMmcs{});
    // out: rounds, roots, final polynomial, query witness, per query its index and per round the
    // siblings and the path, then the challenger afterwards
    std::vector<unsigned char> out;
    auto put32 = [&](uint32_t v) { out.insert(out.end(), reinterpret_cast<unsigned char*>(&v), reinterpret_cast<unsigned char*>(&v) + 4); };
    auto put64 = [&](uint64_t v) { out.insert(out.end(), reinterpret_cast<unsigned char*>(&v), reinterpret_cast<unsigned char*>(&v) + 8); };
    put32(uint32_t(proof.commit_phase_commits.size()));
    for (const auto& c : proof.commit_phase_commits)
        for (const auto& e : c.at(0)) put32(e.value());
    put32(uint32_t(proof.final_poly.size()));
    for (const auto& v : proof.final_poly)
        for (int e = 0; e < 4; ++e) put32(v[e].value());
    put64(proof.query_pow_witness);
    put32(uint32_t(proof.query_proofs.size()));
    for (const auto& qp : proof.query_proofs) {
        put64(qp.input_proof.row_index);
        for (const auto& step : qp.commit_phase_openings) {
            put32(step.log_arity);
            put32(uint32_t(step.sibling_values.size()));
            for (const auto& v : step.sibling_values)
                for (int e = 0; e < 4; ++e) put32(v[e].value());
            put32(uint32_t(step.opening_proof.size()));
            for (const auto& d : step.opening_proof)
                for (const auto& e : d) put32(e.value());
        }
    }
    const p3g_challenger after = tr.inner.state();
    const unsigned char* ab = reinterpret_cast<const unsigned char*>(&after);
    out.insert(out.end(), ab, ab + sizeof after);
    write_file(a[3], out);
    return 0;
}

template <class F>
static int run_lde(char** a) {
    auto in = read_file(a[3]);
    const size_t log_h = std::strtoul(a[5], nullptr, 0), w = std::strtoul(a[6], nullptr, 0);
    const size_t bits = std::strtoul(a[7], nullptr, 0);
    const uint64_t shift = std::strtoull(a[8], nullptr, 0);
    RowMajorMatrix<F> m(p3g::from_words<F>(in.data(), (size_t(1) << log_h) * w), w);
    p3g::GpuDft<Radix2Dit> dft;
    auto out = dft.coset_lde_batch(std::move(m), bits, F(shift));
    write_file(a[4], p3g::to_words(out.values));
    return 0;
}

template <class F>
static int run_dft(char** a) {
    auto in = read_file(a[3]);
    const size_t log_h = std::strtoul(a[5], nullptr, 0), w = std::strtoul(a[6], nullptr, 0);
    const int kind = std::atoi(a[7]);
    const F shift(std::strtoull(a[8], nullptr, 0));
    RowMajorMatrix<F> m(p3g::from_words<F>(in.data(), (size_t(1) << log_h) * w), w);
    p3g::GpuDft<Radix2Dit> dft;
    RowMajorMatrix<F> out = kind == 0   ? dft.dft_batch(std::move(m))
                            : kind == 1 ? dft.idft_batch(std::move(m))
                            : kind == 2 ? dft.coset_dft_batch(std::move(m), shift)
                                        : dft.coset_idft_batch(std::move(m), shift);
    write_file(a[4], p3g::to_words(out.values));
    return 0;
}

template <class F, size_t N>
static int run_mmcs(int argc, char** a) {
    auto in = read_file(a[3]);
    const size_t cap = std::strtoul(a[5], nullptr, 0);
    constexpr size_t E = sizeof(F) == 4 ? 4 : 8;
    std::vector<RowMajorMatrix<F>> mats;
    size_t off = 0;
    for (int i = 6; i + 1 < argc; i += 2) {
        const size_t h = std::strtoul(a[i], nullptr, 0), w = std::strtoul(a[i + 1], nullptr, 0);
        mats.emplace_back(p3g::from_words<F>(in.data() + off, h * w), w);
        off += h * w * E;
    }
    using M = MixedMmcs<F, N>;
    p3g::GpuMerkleTreeMmcs<M> mmcs(typename M::Sponge{}, typename M::Trunc{}, cap);
    auto [commitment, pd] = mmcs.commit(std::move(mats));
    std::vector<unsigned char> out;
    append_layers(out, pd.digest_layers);
    if (commitment.cap != pd.digest_layers.back()) return 3;
    write_file(a[4], out);
    return 0;
}

// build_merkle_tree_cuda with the seeded constants in a Poseidon2Cuda-like struct
template <class F>
static int run_build_tree(int argc, char** a) {
    auto in = read_file(a[3]);
    const size_t cap = std::strtoul(a[5], nullptr, 0);
    constexpr size_t E = sizeof(F);
    std::vector<RowMajorMatrix<F>> mats;
    size_t off = 0;
    for (int i = 6; i + 1 < argc; i += 2) {
        const size_t h = std::strtoul(a[i], nullptr, 0), w = std::strtoul(a[i + 1], nullptr, 0);
        mats.emplace_back(p3g::from_words<F>(in.data() + off, h * w), w);
        off += h * w * E;
    }
    std::vector<unsigned char> out;
    if constexpr (E == 4) {
        Poseidon2Cuda<F, 16, 8, 13, 7> pos;
        std::mt19937 r32(0xdeadbeef);
        for (size_t r = 0; r < 4; ++r)
            for (size_t i = 0; i < 16; ++i) {
                pos.initial_external_constants[r][i] = F(uint32_t(r32() % F::PRIME));
                pos.terminal_external_constants[r][i] = F(uint32_t(r32() % F::PRIME));
            }
        for (size_t r = 0; r < 13; ++r) pos.internal_constants[r] = F(uint32_t(r32() % F::PRIME));
        auto tree = p3g::build_merkle_tree_cuda<F, 16, 8, 8, 8, 13, 7>(std::move(mats), pos, cap);
        append_layers(out, tree.digest_layers);
    } else {
        Poseidon2Cuda<F, 8, 8, 22, 7> pos;
        std::mt19937_64 r64(12345);
        for (size_t r = 0; r < 4; ++r)
            for (size_t i = 0; i < 8; ++i) {
                pos.initial_external_constants[r][i] = F(r64() % F::PRIME);
                pos.terminal_external_constants[r][i] = F(r64() % F::PRIME);
            }
        for (size_t r = 0; r < 22; ++r) pos.internal_constants[r] = F(r64() % F::PRIME);
        auto tree = p3g::build_merkle_tree_cuda<F, 8, 4, 4, 8, 22, 7>(std::move(mats), pos, cap);
        append_layers(out, tree.digest_layers);
    }
    write_file(a[4], out);
    return 0;
}

// TwoAdicFriPcs::commit (two_adic_fri_pcs.hpp:207-266) as the PCS chains its
// members: GpuDft::coset_lde_batch per matrix (natural order, the domain's
// shift), the rows of every LDE side by side with row r of a shorter LDE
// taken as r mod its height, the width padded with zero columns to a power of
// two, then GpuInputMmcs::commit_matrix of that flat matrix.
static int run_pcs_commit(int argc, char** a) {
    if (argc < 8 || (argc - 6) % 2) return 2;
    auto in = read_file(a[2]);
    const size_t log_blowup = std::strtoul(a[4], nullptr, 0);
    const BabyBear shift(uint32_t(std::strtoul(a[5], nullptr, 0)));
    p3g::GpuDft<Radix2Dit> dft;
    std::vector<RowMajorMatrix<BabyBear>> ldes;
    size_t off = 0;
    for (int i = 6; i + 1 < argc; i += 2) {
        const size_t h = size_t(1) << std::strtoul(a[i], nullptr, 0), w = std::strtoul(a[i + 1], nullptr, 0);
        RowMajorMatrix<BabyBear> m(p3g::from_words<BabyBear>(in.data() + off, h * w), w);
        off += 4 * h * w;
        ldes.push_back(dft.coset_lde_batch(std::move(m), log_blowup, shift));
    }
    size_t max_h = 0, total_w = 0;
    for (const auto& l : ldes) {
        max_h = std::max(max_h, l.height());
        total_w += l.width();
    }
    size_t padded_w = 1;
    while (padded_w < total_w) padded_w <<= 1;
    std::vector<BabyBear> flat;
    flat.reserve(max_h * padded_w);
    for (size_t r = 0; r < max_h; ++r) {
        for (const auto& l : ldes) {
            const size_t row = r % l.height();
            flat.insert(flat.end(), l.values.begin() + row * l.width(), l.values.begin() + (row + 1) * l.width());
        }
        flat.resize(flat.size() + (padded_w - total_w), BabyBear(0));
    }
    p3g::GpuInputMmcs<FlatMmcs<BabyBear, 8>> mmcs{FlatMmcs<BabyBear, 8>{}};
    auto [commitment, pd] = mmcs.commit_matrix(flat, padded_w);
    if (commitment.size() != 1 || pd.height != max_h || pd.width != padded_w) return 3;
    std::vector<BabyBear> out(commitment[0].begin(), commitment[0].end());
    out.insert(out.end(), flat.begin(), flat.end());
    write_file(a[3], p3g::to_words(out));
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    const std::string cmd = argv[1];
    try {
        set_constants();
        if (cmd == "challenger") return run_challenger(argc, argv);
        if (cmd == "prove_fri") return run_prove_fri(argc, argv);
        if (cmd == "pcs_commit") return run_pcs_commit(argc, argv);
        if (cmd == "lde") return std::string(argv[2]) == "bb" ? run_lde<BabyBear>(argv) : run_lde<Goldilocks>(argv);
        if (cmd == "dft") {
            if (argc < 9) return 2;
            return std::string(argv[2]) == "bb" ? run_dft<BabyBear>(argv) : run_dft<Goldilocks>(argv);
        }
        if (cmd == "build_tree")
            return std::string(argv[2]) == "bb" ? run_build_tree<BabyBear>(argc, argv)
                                                : run_build_tree<Goldilocks>(argc, argv);
        if (cmd == "mmcs")
            return std::string(argv[2]) == "bb" ? run_mmcs<BabyBear, 8>(argc, argv) : run_mmcs<Goldilocks, 4>(argc, argv);
        if (cmd == "commit_matrix") {
            auto in = read_file(argv[2]);
            const size_t h = std::strtoul(argv[4], nullptr, 0), w = std::strtoul(argv[5], nullptr, 0);
            p3g::GpuInputMmcs<FlatMmcs<BabyBear, 8>> mmcs{FlatMmcs<BabyBear, 8>{}};
            auto [commitment, pd] = mmcs.commit_matrix(p3g::from_words<BabyBear>(in.data(), h * w), w);
            if (pd.height != h || pd.width != w || commitment.size() != 1) return 3;
            std::vector<unsigned char> out;
            append_layers(out, pd.tree);
            write_file(argv[3], out);
            return 0;
        }
        if (cmd == "fold_cuda") {  // fold_matrix_cuda (host) and fold_matrix_cuda_device must agree
            auto in = read_file(argv[2]);
            const size_t log_h = std::strtoul(argv[4], nullptr, 0), la = std::strtoul(argv[5], nullptr, 0);
            auto words = p3g::from_words<BabyBear>(in.data(), 4 + (size_t(4) << log_h));
            BabyBear4 beta;
            for (int k = 0; k < 4; ++k) beta[k] = words[k];
            std::vector<BabyBear4> cur(size_t(1) << log_h);
            for (size_t i = 0; i < cur.size(); ++i)
                for (int k = 0; k < 4; ++k) cur[i][k] = words[4 + 4 * i + k];
            auto host = p3g::fold_matrix_cuda<BabyBear, BabyBear4>(beta, la, log_h, cur);
            const size_t n = cur.size() >> la;
            p3g::DeviceBuffer din(cur.size() * 16), dout(n * 16);
            din.upload(cur.data(), cur.size() * 16);
            p3g::fold_matrix_cuda_device<BabyBear, BabyBear4>(static_cast<const BabyBear4*>(din.get()),
                                                              static_cast<BabyBear4*>(dout.get()), beta, la, log_h, n);
            std::vector<BabyBear4> dev(n);
            dout.download(dev.data(), n * 16);
            std::vector<BabyBear> flat;
            for (size_t i = 0; i < n; ++i)
                for (int k = 0; k < 4; ++k) {
                    if (!(dev[i][k] == host[i][k])) return 7;
                    flat.push_back(host[i][k]);
                }
            write_file(argv[3], p3g::to_words(flat));
            return 0;
        }
        if (cmd == "fold") {
            auto in = read_file(argv[2]);
            const size_t log_h = std::strtoul(argv[4], nullptr, 0), la = std::strtoul(argv[5], nullptr, 0);
            auto words = p3g::from_words<BabyBear>(in.data(), 4 + (size_t(4) << log_h));
            BabyBear4 beta;
            for (int k = 0; k < 4; ++k) beta[k] = words[k];
            std::vector<BabyBear4> cur(size_t(1) << log_h);
            for (size_t i = 0; i < cur.size(); ++i)
                for (int k = 0; k < 4; ++k) cur[i][k] = words[4 + 4 * i + k];
            auto res = p3g::gpu_fold_matrix<BabyBear, BabyBear4>(log_h, la, beta, cur);
            std::vector<BabyBear> flat;
            for (const auto& e : res)
                for (int k = 0; k < 4; ++k) flat.push_back(e[k]);
            write_file(argv[3], p3g::to_words(flat));
            return 0;
        }
    } catch (const std::invalid_argument& e) {
        std::fprintf(stderr, "invalid_argument: %s\n", e.what());
        return 4;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 5;
    }
    return 2;
}
