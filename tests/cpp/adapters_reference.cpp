// adapters_reference.cpp -- the reference's own prover types with the GPU
// adapters swapped in, checked against the same types without them.
//
// Built against the reference's unmodified headers (dloghin/plonky3-gpu,
// src/include) and libp3g_gb300.so; the CPU test suite compiles and links it
// to show that the adapters drop into TwoAdicFriPcs, MerkleTreeMmcs and
// TwoAdicFriFolding unchanged.  Run on a machine with a GPU it prints one
// line per check and exits non-zero on any mismatch:
//   1. TwoAdicFriPcs<BB, BB4, GpuDft<Radix2Dit>, GpuInputMmcs<flat MMCS>, ...>::commit
//      against the stock Pcs (same commitment), and its open with the FRI MMCS
//      ExtensionMmcs<..., GpuInputMmcs<...>> (same opened values and proof);
//   2. GpuMerkleTreeMmcs<mixed-height MMCS>::commit against the stock one (all
//      digest layers), then the stock open_batch / verify_batch on the GPU tree;
//   3. GpuDft's dft / idft / coset_dft / coset_idft against Radix2Dit's, and
//      GpuDft over the reference's NttCuda;
//   4. gpu_fold_matrix against TwoAdicFriFolding<BB, BB4>::fold_matrix;
//   5. GpuDuplexChallenger against DuplexChallenger: the same observations,
//      samples, sample_bits and grind witnesses;
//   6. gpu_prove_fri against prove_fri: the same FriProof (byte for byte in
//      p3g_proof.hpp's format) and the same transcript afterwards.

#include "baby_bear.hpp"
#include "extension_field.hpp"
#include "dense_matrix.hpp"
#include "radix2_dit.hpp"
#include "ntt_cuda.hpp"
#include "util.hpp"
#include "poseidon2_cuda.hpp"
#include "padding_free_sponge.hpp"
#include "truncated_permutation.hpp"
#include "merkle_tree_mmcs.hpp"
#include "merkle_tree_cuda.hpp"
#include "fri_merkle_tree_mmcs.hpp"
#include "fri_extension_mmcs.hpp"
#include "fri_folding.hpp"
#include "fri_params.hpp"
#include "two_adic_fri_pcs.hpp"
#include "duplex_challenger.hpp"
#include "fri_prover.hpp"

#include "p3g_adapters.hpp"
#include "p3g_proof.hpp"

#include <cstdio>
#include <random>

using namespace p3_field;
using p3_matrix::RowMajorMatrix;
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
using Mixed = p3_merkle_tree::MerkleTreeMmcs<BB, BB, Sponge, Trunc, 8>;
using EFMmcs = p3_merkle::ExtensionMmcs<BB, BabyBear4, Flat>;

static RowMajorMatrix<BB> rand_matrix(size_t h, size_t w, uint32_t seed) {
    std::mt19937 rng(seed);
    std::vector<BB> v(h * w);
    for (auto& e : v) e = BB(uint32_t(rng() % BB::PRIME));
    return RowMajorMatrix<BB>(std::move(v), w);
}

// prove_fri's input MMCS for check 6: the opening records the index.
struct IndexMmcs {
    struct ProverData {};
    struct OpeningProof {
        size_t row_index = 0;
        std::vector<BB> row_values;
    };
    void open(size_t index, const std::vector<ProverData>&, OpeningProof& p) const { p.row_index = index; }
};
template <class Inner>
struct FriTranscript {  // the FRI tests' wrapper (fri_test.cpp:100-120)
    Inner inner;
    template <typename C>
    void observe_commitment(const C& c) { inner.observe_merkle_cap(c); }
    template <typename EF = BabyBear4>
    EF sample_challenge() { return inner.template sample_algebra_element<EF>(); }
    template <typename EF>
    void observe_challenge(const EF& v) { inner.template observe_algebra_element<EF>(v); }
    void observe_arity(size_t la) { inner.observe(BB(static_cast<uint32_t>(la))); }
    uint64_t grind(size_t bits) { return inner.grind(bits); }
    bool check_witness(size_t bits, uint64_t w) { return inner.check_witness(bits, w); }
    size_t sample_bits(size_t n) { return inner.sample_bits(n); }
};

static int report(const char* what, bool ok) {
    std::printf("%s %s\n", ok ? "ok  " : "FAIL", what);
    return ok ? 0 : 1;
}

int main() {
    int fails = 0;
    const Pos pos = make_pos();
    p3g::Context::get().set_poseidon2(pos.initial_external_constants, pos.terminal_external_constants,
                                      pos.internal_constants, 7);
    auto flat = [&] { return Flat(Sponge(Wrap{pos}), Trunc(Wrap{pos})); };
    const std::vector<std::pair<size_t, size_t>> shapes = {{10, 7}, {8, 3}, {10, 2}, {6, 5}};

    // 1. PCS commit
    {
        using Cpu = p3_fri::TwoAdicFriPcs<BB, BabyBear4, p3_dft::Radix2Dit<BB>, Flat, EFMmcs>;
        using Gpu = p3_fri::TwoAdicFriPcs<BB, BabyBear4, p3g::GpuDft<p3_dft::Radix2Dit<BB>>, p3g::GpuInputMmcs<Flat>,
                                          EFMmcs>;
        p3_fri::FriParameters<EFMmcs> fri_a{1, 0, 1, 10, 0, 8, EFMmcs(flat())};
        p3_fri::FriParameters<EFMmcs> fri_b{1, 0, 1, 10, 0, 8, EFMmcs(flat())};
        Cpu cpu(p3_dft::Radix2Dit<BB>(), flat(), std::move(fri_a));
        Gpu gpu(p3g::GpuDft<p3_dft::Radix2Dit<BB>>(), p3g::GpuInputMmcs<Flat>(flat()), std::move(fri_b));
        auto evals = [&](auto& pcs) {
            std::vector<std::pair<typename std::decay_t<decltype(pcs)>::Domain, RowMajorMatrix<BB>>> ev;
            for (size_t i = 0; i < shapes.size(); ++i) {
                typename std::decay_t<decltype(pcs)>::Domain d;
                d.log_n = shapes[i].first;
                d.shift = BB::one_val();
                ev.push_back({d, rand_matrix(size_t(1) << shapes[i].first, shapes[i].second, 100 + uint32_t(i))});
            }
            return ev;
        };
        auto [c_cpu, pd_cpu] = cpu.commit(evals(cpu));
        auto [c_gpu, pd_gpu] = gpu.commit(evals(gpu));
        fails += report("TwoAdicFriPcs::commit with GpuDft + GpuInputMmcs", c_cpu == c_gpu);

        // the reference's own open / prove_fri with every FRI round committed on the GPU
        // (ExtensionMmcs over GpuInputMmcs as the FRI MMCS)
        using GpuEF = p3_merkle::ExtensionMmcs<BB, BabyBear4, p3g::GpuInputMmcs<Flat>>;
        using GpuFri = p3_fri::TwoAdicFriPcs<BB, BabyBear4, p3g::GpuDft<p3_dft::Radix2Dit<BB>>,
                                             p3g::GpuInputMmcs<Flat>, GpuEF>;
        p3_fri::FriParameters<GpuEF> fri_c{1, 0, 1, 10, 0, 8, GpuEF(p3g::GpuInputMmcs<Flat>(flat()))};
        GpuFri gpu_fri(p3g::GpuDft<p3_dft::Radix2Dit<BB>>(), p3g::GpuInputMmcs<Flat>(flat()), std::move(fri_c));
        auto [c_fri, pd_fri] = gpu_fri.commit(evals(gpu_fri));
        using Tr = FriTranscript<p3_challenger::DuplexChallenger<BB, Wrap, 16, 8>>;
        auto open = [&](auto& pcs, const auto& commit, const auto& pd) {
            Tr t{p3_challenger::DuplexChallenger<BB, Wrap, 16, 8>(Wrap{pos})};
            t.observe_commitment(commit);
            const BabyBear4 z = t.template sample_challenge<BabyBear4>();
            std::vector<std::vector<BabyBear4>> pts(shapes.size(), std::vector<BabyBear4>{z});
            auto [ov, proof] = pcs.open({{&pd, pts}}, t);
            return std::make_pair(p3g::wire::encode(ov), p3g::wire::encode(proof));
        };
        fails += report("TwoAdicFriPcs::open with GPU-committed FRI rounds: the same opened values and proof",
                        open(cpu, c_cpu, pd_cpu) == open(gpu_fri, c_fri, pd_fri));
    }

    // 2. mixed-height MMCS commit, then the stock opening and verification
    {
        Mixed cpu(Sponge(Wrap{pos}), Trunc(Wrap{pos}), 1);
        p3g::GpuMerkleTreeMmcs<Mixed> gpu(Sponge(Wrap{pos}), Trunc(Wrap{pos}), 1);
        auto mats = [&] {
            std::vector<RowMajorMatrix<BB>> m;
            for (size_t i = 0; i < shapes.size(); ++i)
                m.push_back(rand_matrix(size_t(1) << shapes[i].first, shapes[i].second, 200 + uint32_t(i)));
            return m;
        };
        auto [cap_cpu, tree_cpu] = cpu.commit(mats());
        auto [cap_gpu, tree_gpu] = gpu.commit(mats());
        fails += report("MerkleTreeMmcs::commit digest layers", tree_cpu.digest_layers == tree_gpu.digest_layers &&
                                                                    cap_cpu == cap_gpu);
        bool ok = true;
        std::vector<p3_matrix::Dimensions> dims;
        for (const auto& m : tree_gpu.leaves) dims.push_back({m.width(), m.height()});
        for (size_t index : {size_t(0), size_t(1), size_t(517), size_t(1023)}) {
            auto opening = gpu.open_batch(index, tree_gpu);
            ok = ok && cpu.verify_batch(cap_gpu, dims, index, opening);
        }
        fails += report("open_batch on the GPU tree verifies", ok);
        // the reference's GPU tree-build signature (its CPU fallback in this build)
        auto want = p3_merkle_tree::build_merkle_tree_cuda<BB, 16, 8, 8, 8, 13, 7>(mats(), pos, 1);
        auto got = p3g::build_merkle_tree_cuda<BB, 16, 8, 8, 8, 13, 7>(mats(), pos, 1);
        fails += report("build_merkle_tree_cuda digest layers", want.digest_layers == got.digest_layers);
    }

    // 3. the other Dft members against Radix2Dit
    {
        p3_dft::Radix2Dit<BB> cpu;
        p3g::GpuDft<p3_dft::Radix2Dit<BB>> gpu;
        const BB shift(uint32_t(7));
        bool ok = true;
        for (size_t log_h : {size_t(3), size_t(10), size_t(13)}) {
            auto m = [&] { return rand_matrix(size_t(1) << log_h, 5, 300 + uint32_t(log_h)); };
            ok = ok && cpu.dft_batch(m()).values == gpu.dft_batch(m()).values;
            ok = ok && cpu.idft_batch(m()).values == gpu.idft_batch(m()).values;
            ok = ok && cpu.coset_dft_batch(m(), shift).values == gpu.coset_dft_batch(m(), shift).values;
            ok = ok && cpu.coset_idft_batch(m(), shift).values == gpu.coset_idft_batch(m(), shift).values;
        }
        fails += report("dft_batch / idft_batch / coset_dft_batch / coset_idft_batch", ok);
        // the same adapter over the reference's own GPU NTT class
        p3g::GpuDft<p3_dft::NttCuda<BB>> gpu_ntt;
        auto m = [&] { return rand_matrix(size_t(1) << 12, 6, 400); };
        bool ok2 = cpu.coset_lde_batch(m(), 1, BB(uint32_t(31))).values ==
                       gpu_ntt.coset_lde_batch(m(), 1, BB(uint32_t(31))).values &&
                   cpu.dft_batch(m()).values == gpu_ntt.dft_batch(m()).values;
        fails += report("GpuDft<NttCuda<BabyBear>> in place of NttCuda", ok2);
    }

    // 4. fold_matrix
    {
        std::mt19937 rng(7);
        auto r = [&] { return BB(uint32_t(rng() % BB::PRIME)); };
        for (size_t la = 1; la <= 3; ++la) {
            const size_t log_h = 11;
            std::vector<BabyBear4> v(size_t(1) << log_h);
            for (auto& e : v) e = BabyBear4({r(), r(), r(), r()});
            const BabyBear4 beta({r(), r(), r(), r()});
            auto want = p3_fri::TwoAdicFriFolding<BB, BabyBear4>::fold_matrix(log_h, la, beta, v);
            auto got = p3g::gpu_fold_matrix<BB, BabyBear4>(log_h, la, beta, v);
            auto got_cuda = p3g::fold_matrix_cuda<BB, BabyBear4>(beta, la, log_h, v);  // fri_fold_cuda.hpp's order
            fails += report(la == 1 ? "fold_matrix arity 2" : la == 2 ? "fold_matrix arity 4" : "fold_matrix arity 8",
                            want == got && want == got_cuda);
        }
    }
    // 5. the challenger
    {
        p3_challenger::DuplexChallenger<BB, Wrap, 16, 8> cpu(Wrap{pos});
        p3g::GpuDuplexChallenger<BB, Wrap, 16, 8> gpu(Wrap{pos});
        std::mt19937 rng(11);
        bool ok = true;
        for (size_t n_obs : {size_t(3), size_t(7), size_t(6), size_t(1)}) {
            for (size_t i = 0; i < n_obs; ++i) {
                const BB v(uint32_t(rng() % BB::PRIME));
                cpu.observe(v);
                gpu.observe(v);
            }
            for (size_t bits : {size_t(0), size_t(9), size_t(14)}) ok = ok && cpu.grind(bits) == gpu.grind(bits);
            ok = ok && cpu.sample() == gpu.sample() && cpu.sample_bits(20) == gpu.sample_bits(20);
            const auto a = cpu.sample_algebra_element<BabyBear4>();
            const auto b = gpu.sample_algebra_element<BabyBear4>();
            ok = ok && a == b;
            cpu.observe_algebra_element(a);
            gpu.observe_algebra_element(b);
        }
        p3g::GpuDuplexChallenger<BB, Wrap, 16, 8> resumed(Wrap{pos});
        resumed.set_state(gpu.state());
        for (int k = 0; k < 10; ++k) ok = ok && resumed.sample() == cpu.sample();
        fails += report("DuplexChallenger with grind on the GPU", ok);
    }
    // 6. prove_fri with the data and the transcript on the GPU
    {
        using Cpu = FriTranscript<p3_challenger::DuplexChallenger<BB, Wrap, 16, 8>>;
        using Gpu = FriTranscript<p3g::GpuDuplexChallenger<BB, Wrap, 16, 8>>;
        Cpu cpu{p3_challenger::DuplexChallenger<BB, Wrap, 16, 8>(Wrap{pos})};
        Gpu gpu{p3g::GpuDuplexChallenger<BB, Wrap, 16, 8>(Wrap{pos})};
        std::mt19937 rng(13);
        auto r = [&] { return BB(uint32_t(rng() % BB::PRIME)); };
        std::vector<std::vector<BabyBear4>> inputs;
        for (size_t lh : {size_t(11), size_t(9), size_t(6)}) {
            std::vector<BabyBear4> v(size_t(1) << lh);
            for (auto& e : v) e = BabyBear4({r(), r(), r(), r()});
            inputs.push_back(std::move(v));
        }
        p3_fri::FriParameters<EFMmcs> fp{1, 1, 3, 20, 4, 10, EFMmcs(flat())};
        std::vector<IndexMmcs::ProverData> none;
        auto want = p3_fri::prove_fri<BB, BabyBear4, EFMmcs, Cpu, uint64_t, IndexMmcs, IndexMmcs::OpeningProof>(
            fp, inputs, cpu, none, IndexMmcs{});
        auto got = p3g::gpu_prove_fri<BB, BabyBear4, EFMmcs, Gpu, uint64_t, IndexMmcs, IndexMmcs::OpeningProof>(
            fp, inputs, gpu, none, IndexMmcs{});
        bool ok = p3g::wire::encode(want) == p3g::wire::encode(got);
        for (int k = 0; k < 8; ++k) ok = ok && cpu.inner.sample() == gpu.inner.sample();
        fails += report("gpu_prove_fri: the same FriProof and transcript as prove_fri", ok);
    }
    std::printf("%s\n", fails ? "MISMATCH" : "ALL OK");
    return fails ? 1 : 0;
}
