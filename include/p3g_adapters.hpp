// p3g_adapters.hpp -- drop-in C++ adapters for the reference's commitment interfaces.
//
// Each adapter derives from the reference class it accelerates and replaces
// only the hot member with a call through the C ABI (p3g.h); everything else
// -- openings, verification, the Commitment / ProverData types -- is the
// reference's own.  Host data in, host data out, exactly like the reference
// (by-value RowMajorMatrix, host copies of leaves and digest layers), so the
// adapters can be passed as template arguments wherever the reference classes
// are:
//
//   GpuDft<p3_dft::Radix2Dit<BabyBear>>            coset_lde_batch      (radix2_dit.hpp:221),
//                                                  dft_batch, idft_batch, coset_dft_batch,
//                                                  coset_idft_batch     (radix2_dit.hpp:82-210)
//   GpuInputMmcs<p3_merkle::MerkleTreeMmcs<...>>   commit_matrix        (fri_merkle_tree_mmcs.hpp:55)
//   GpuMerkleTreeMmcs<p3_merkle_tree::MerkleTreeMmcs<...>> commit       (merkle_tree_mmcs.hpp:100)
//   gpu_fold_matrix<Val, Challenge>(...)          fold_matrix           (fri_folding.hpp:200)
//   fold_matrix_cuda / fold_matrix_cuda_device     the reference's GPU fold (fri_fold_cuda.hpp:250-348)
//   build_merkle_tree_cuda<F, WIDTH, RATE, ...>    the reference's GPU tree build (merkle_tree_cuda.hpp:358)
//   gpu_prove_fri<Val, Challenge, ...>(...)        prove_fri, data and transcript on the GPU
//                                                  (fri_prover.hpp:35-265)
//   GpuDuplexChallenger<F, Perm, WIDTH, RATE>     DuplexChallenger with grind on the GPU
//                                                  (duplex_challenger.hpp:42-285)
//
// e.g. TwoAdicFriPcs<BB, BB4, GpuDft<Radix2Dit<BB>>, GpuInputMmcs<FlatMmcs>, EFMmcs>.
// The element types must be the reference's 4-byte BabyBear (value(),
// BabyBear(uint32_t)) or 8-byte Goldilocks (as_canonical_u64(),
// Goldilocks(uint64_t)); a BabyBear4 challenge exposes operator[] over 4
// BabyBear coefficients.  Errors raise std::invalid_argument (bad arguments,
// as the reference's log2_strict_usize does) or std::runtime_error (device
// failures).  All calls use the process-wide p3g::Context.
#pragma once

#include <algorithm>
#include <array>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "p3g.h"

namespace p3_merkle_tree {  // the reference's tree type (merkle_tree.hpp:45-58), for build_merkle_tree_cuda
template <typename F, typename W, size_t DIGEST_ELEMS>
struct MerkleTree;
}  // namespace p3_merkle_tree
namespace p3_fri {  // the reference's FRI types (fri_params.hpp:9-24, fri_proof.hpp:25-32), for gpu_prove_fri
template <typename FriMmcs>
struct FriParameters;
template <typename Challenge, typename FriMmcs, typename Witness, typename InputProof>
struct FriProof;
}  // namespace p3_fri

namespace p3g {

inline void check(int status) {
    if (status == P3G_OK) return;
    char msg[1024];
    p3g_last_error(msg, sizeof msg);
    if (status == P3G_EINVAL) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

template <class F>
constexpr int field_id() {
    static_assert(sizeof(F) == 4 || sizeof(F) == 8, "BabyBear (4 bytes) or Goldilocks (8 bytes)");
    return sizeof(F) == 4 ? P3G_BABYBEAR : P3G_GOLDILOCKS;
}
template <class F>
inline uint64_t canonical(const F& x) {
    if constexpr (sizeof(F) == 4) return uint64_t(x.value());
    else return x.as_canonical_u64();
}
template <class F>
inline F from_canonical(uint64_t v) {
    if constexpr (sizeof(F) == 4) return F(uint32_t(v));
    else return F(uint64_t(v));
}

// Process-wide context (device 0 unless select_device() runs first).
class Context {
   public:
    static Context& get() {
        static Context c;
        return c;
    }
    void select_device(int d) { device_ = d; }
    p3g_ctx* handle() {
        std::lock_guard<std::mutex> lk(mu_);
        if (!ctx_) check(p3g_ctx_create(device_, &ctx_));
        return ctx_;
    }
    // Poseidon2 constants in the reference's constructor shape (poseidon2.hpp:193):
    // ExternalLayerConstants' initial / terminal rows and the internal constants.
    template <class F, size_t W>
    void set_poseidon2(const std::vector<std::array<F, W>>& initial, const std::vector<std::array<F, W>>& terminal,
                       const std::vector<F>& internal, uint32_t degree) {
        if (initial.size() != terminal.size()) throw std::invalid_argument("External constants size mismatch");
        std::vector<uint64_t> ini, ter, inr;
        for (size_t r = 0; r < initial.size(); ++r)
            for (size_t i = 0; i < W; ++i) {
                ini.push_back(canonical(initial[r][i]));
                ter.push_back(canonical(terminal[r][i]));
            }
        for (const F& c : internal) inr.push_back(canonical(c));
        if (inr.empty()) inr.push_back(0);
        const uint32_t rf = uint32_t(2 * initial.size()), rp = uint32_t(internal.size());
        if constexpr (sizeof(F) == 4) {
            std::vector<uint32_t> a(ini.begin(), ini.end()), b(ter.begin(), ter.end()), c(inr.begin(), inr.end());
            check(p3g_set_poseidon2(handle(), P3G_BABYBEAR, uint32_t(W), rf, rp, degree, a.data(), b.data(), c.data()));
        } else {
            check(p3g_set_poseidon2(handle(), P3G_GOLDILOCKS, uint32_t(W), rf, rp, degree, ini.data(), ter.data(),
                                    inr.data()));
        }
    }
    // The same from a Poseidon2Cuda<F, W, RF, RP, D> (poseidon2_cuda.hpp:38).
    template <class F, size_t W, size_t RF, size_t RP>
    void set_poseidon2(const F (&initial)[RF][W], const F (&terminal)[RF][W], const F (&internal)[RP],
                       uint32_t degree) {
        std::vector<std::array<F, W>> a(RF), b(RF);
        for (size_t r = 0; r < RF; ++r)
            for (size_t i = 0; i < W; ++i) {
                a[r][i] = initial[r][i];
                b[r][i] = terminal[r][i];
            }
        set_poseidon2(a, b, std::vector<F>(internal, internal + RP), degree);
    }
    ~Context() {
        if (ctx_) p3g_ctx_destroy(ctx_);
    }

   private:
    Context() = default;
    std::mutex mu_;
    int device_ = 0;
    p3g_ctx* ctx_ = nullptr;
};

// Device buffer from the context pool.
class DeviceBuffer {
   public:
    explicit DeviceBuffer(size_t bytes) : ctx_(Context::get().handle()) { check(p3g_malloc(ctx_, bytes, &p_, nullptr)); }
    ~DeviceBuffer() {
        if (p_) p3g_free(ctx_, p_, nullptr);
    }
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    void* get() const { return p_; }
    void upload(const void* h, size_t bytes) { check(p3g_memcpy_h2d(ctx_, p_, h, bytes, nullptr)); }
    void download(void* h, size_t bytes) const { check(p3g_memcpy_d2h(ctx_, h, p_, bytes, nullptr)); }

   private:
    p3g_ctx* ctx_;
    void* p_ = nullptr;
};

// Canonical words of a field vector (u32 for BabyBear, u64 for Goldilocks).
template <class F>
inline std::vector<unsigned char> to_words(const std::vector<F>& v) {
    constexpr size_t E = sizeof(F) == 4 ? 4 : 8;
    std::vector<unsigned char> out(v.size() * E);
    for (size_t i = 0; i < v.size(); ++i) {
        const uint64_t c = canonical(v[i]);
        std::memcpy(out.data() + i * E, &c, E);  // little-endian low bytes
    }
    return out;
}
template <class F>
inline std::vector<F> from_words(const unsigned char* p, size_t n) {
    constexpr size_t E = sizeof(F) == 4 ? 4 : 8;
    std::vector<F> out;
    out.reserve(n);
    for (size_t i = 0; i < n; ++i) {
        uint64_t c = 0;
        std::memcpy(&c, p + i * E, E);
        out.push_back(from_canonical<F>(c));
    }
    return out;
}

// Host copy of every digest layer of a device tree, in the reference's
// vector-of-layers shape (layer 0 = leaf digests, last = cap).
template <class Dg>
std::vector<std::vector<Dg>> download_layers(p3g_ctx* ctx, const p3g_tree* tree) {
    using W = std::decay_t<decltype(std::declval<Dg&>()[0])>;
    uint32_t nl = 0, dig = 0;
    uint64_t sizes[64];
    check(p3g_tree_info(tree, &nl, sizes, &dig));
    if (dig != std::tuple_size<Dg>::value) throw std::invalid_argument("digest length mismatch");
    constexpr size_t E = sizeof(W) == 4 ? 4 : 8;
    std::vector<std::vector<Dg>> layers(nl);
    for (uint32_t l = 0; l < nl; ++l) {
        const void* dp = nullptr;
        check(p3g_tree_layer_ptr(tree, l, &dp));
        std::vector<unsigned char> raw(sizes[l] * dig * E);
        check(p3g_memcpy_d2h(ctx, raw.data(), dp, raw.size(), nullptr));
        auto flat = from_words<W>(raw.data(), sizes[l] * dig);
        layers[l].resize(sizes[l]);
        for (uint64_t i = 0; i < sizes[l]; ++i)
            for (uint32_t e = 0; e < dig; ++e) layers[l][i][e] = flat[i * dig + e];
    }
    return layers;
}

inline size_t log2_strict(size_t n) {
    if (n == 0 || (n & (n - 1))) throw std::invalid_argument("log2_strict_usize: value must be a non-zero power of 2");
    size_t k = 0;
    while ((size_t(1) << k) < n) ++k;
    return k;
}

// ----------------------------------------------------------------- Dft
// Radix2Dit-compatible; coset_lde_batch runs on the GPU (natural row order,
// as radix2_dit.hpp:221-233 returns it).
template <class Base>
struct GpuDft : Base {
    using Base::Base;
    GpuDft() = default;
    explicit GpuDft(Base b) : Base(std::move(b)) {}

    template <class Mat, class F>
    Mat coset_lde_batch(Mat mat, size_t added_bits, const F& shift) {
        const size_t h = mat.height(), w = mat.width();
        if (h == 0 || w == 0) return Base::coset_lde_batch(std::move(mat), added_bits, shift);
        const size_t log_h = log2_strict(h);
        constexpr size_t E = sizeof(F) == 4 ? 4 : 8;
        const size_t H = h << added_bits;
        auto words = to_words(mat.values);
        DeviceBuffer din(words.size()), dout(H * w * E);
        din.upload(words.data(), words.size());
        check(p3g_coset_lde(Context::get().handle(), field_id<F>(), din.get(), uint32_t(log_h), uint32_t(w),
                            uint32_t(added_bits), canonical(shift), 0, dout.get(), nullptr));
        std::vector<unsigned char> out(H * w * E);
        dout.download(out.data(), out.size());
        return Mat(from_words<F>(out.data(), H * w), w);
    }

    // The other Dft members (radix2_dit.hpp:82-210), natural row order.
    template <class Mat>
    Mat dft_batch(Mat mat) {
        return transform(P3G_DFT, std::move(mat), 0);
    }
    template <class Mat>
    Mat idft_batch(Mat mat) {
        return transform(P3G_IDFT, std::move(mat), 0);
    }
    template <class Mat, class F>
    Mat coset_dft_batch(Mat mat, const F& shift) {
        return transform(P3G_COSET_DFT, std::move(mat), canonical(shift));
    }
    template <class Mat, class F>
    Mat coset_idft_batch(Mat mat, const F& shift) {
        return transform(P3G_COSET_IDFT, std::move(mat), canonical(shift));
    }

   private:
    template <class Mat>
    static Mat transform(int kind, Mat mat, uint64_t shift) {
        using F = std::decay_t<decltype(mat.values[0])>;
        const size_t h = mat.height(), w = mat.width();
        if (h <= 1 || w == 0) return mat;  // every kind leaves one row unchanged (radix2_dit.hpp:84)
        const size_t log_h = log2_strict(h);
        auto words = to_words(mat.values);
        DeviceBuffer din(words.size()), dout(words.size());
        din.upload(words.data(), words.size());
        check(p3g_dft(Context::get().handle(), field_id<F>(), kind, din.get(), uint32_t(log_h), uint32_t(w), shift, 0,
                      dout.get(), nullptr));
        dout.download(words.data(), words.size());
        return Mat(from_words<F>(words.data(), h * w), w);
    }
};

// ----------------------------------------------------------------- flat MMCS
// p3_merkle::MerkleTreeMmcs-compatible; commit_matrix runs on the GPU and
// fills the reference's ProverData (flat_data, height, width, tree layers).
template <class Base>
struct GpuInputMmcs : Base {
    using Base::Base;
    explicit GpuInputMmcs(Base b) : Base(std::move(b)) {}
    using typename Base::Commitment;
    using typename Base::Digest;
    using typename Base::ProverData;

    template <class InputF>
    std::pair<Commitment, ProverData> commit_matrix(const std::vector<InputF>& data, size_t width) const {
        if (width == 0 || data.size() % width != 0) throw std::invalid_argument("commit_matrix: bad dimensions");
        const size_t height = data.size() / width;
        if (height == 0) throw std::invalid_argument("commit_matrix: empty matrix");
        auto words = to_words(data);
        DeviceBuffer d(words.size());
        d.upload(words.data(), words.size());
        p3g_ctx* ctx = Context::get().handle();
        p3g_tree* tree = nullptr;
        check(p3g_commit_matrix(ctx, field_id<InputF>(), d.get(), height, uint32_t(width), &tree, nullptr, nullptr));
        ProverData pd;
        pd.flat_data = data;
        pd.height = height;
        pd.width = width;
        pd.tree = download_layers<Digest>(ctx, tree);
        check(p3g_tree_free(ctx, tree, nullptr));
        Commitment c = {pd.tree.back()[0]};
        return {std::move(c), std::move(pd)};
    }

};

// ----------------------------------------------------------------- mixed-height MMCS
// p3_merkle_tree::MerkleTreeMmcs-compatible; commit runs on the GPU and
// returns the reference's MerkleCap and MerkleTree (leaves + digest layers).
template <class Base>
struct GpuMerkleTreeMmcs : Base {
    using typename Base::Commitment;
    using typename Base::ProverData;

    template <class Hasher, class Compressor>
    GpuMerkleTreeMmcs(Hasher h, Compressor c, size_t cap_height = 0)
        : Base(std::move(h), std::move(c), cap_height), cap_height_(cap_height) {}

    template <class Mat>
    std::pair<Commitment, ProverData> commit(std::vector<Mat> matrices) {
        using F = std::decay_t<decltype(matrices[0].values[0])>;
        constexpr size_t E = sizeof(F) == 4 ? 4 : 8;
        if (matrices.empty()) throw std::invalid_argument("need at least one matrix");
        std::vector<std::unique_ptr<DeviceBuffer>> bufs;
        std::vector<p3g_matrix> descs;
        for (const auto& m : matrices) {
            auto words = to_words(m.values);
            bufs.emplace_back(new DeviceBuffer(std::max<size_t>(words.size(), E)));
            if (!words.empty()) bufs.back()->upload(words.data(), words.size());
            descs.push_back(p3g_matrix{bufs.back()->get(), uint64_t(m.height()), uint32_t(m.width()), 0});
        }
        p3g_ctx* ctx = Context::get().handle();
        p3g_tree* tree = nullptr;
        check(p3g_mmcs_commit(ctx, field_id<F>(), descs.data(), descs.size(), uint32_t(cap_height_), &tree, nullptr,
                              nullptr));
        ProverData pd;
        using Layer = std::decay_t<decltype(pd.digest_layers[0])>;
        using Dg = typename Layer::value_type;
        pd.digest_layers = download_layers<Dg>(ctx, tree);
        check(p3g_tree_free(ctx, tree, nullptr));
        pd.leaves = std::move(matrices);
        Commitment cap(pd.digest_layers.back());
        return {std::move(cap), std::move(pd)};
    }

   private:
    size_t cap_height_;
};

// ----------------------------------------------------------------- fold
// TwoAdicFriFolding<Val, Challenge>::fold_matrix (fri_folding.hpp:200) on the
// GPU for Val = BabyBear and Challenge = BabyBear4 (or BabyBear, embedded).
template <class Val, class Challenge>
std::vector<Challenge> gpu_fold_matrix(size_t log_height, size_t log_arity, const Challenge& beta,
                                       const std::vector<Challenge>& current) {
    static_assert(sizeof(Val) == 4, "fold runs over BabyBear");
    const size_t arity = size_t(1) << log_arity;
    if (current.size() % arity != 0)
        throw std::invalid_argument("fold_matrix: current.size() not divisible by arity");
    if (current.size() != (size_t(1) << log_height))
        throw std::invalid_argument("fold_matrix: current.size() must be 2^log_height");
    constexpr bool EXT = sizeof(Challenge) == 16;
    auto coeff = [](const Challenge& c, int k) -> uint32_t {
        if constexpr (EXT) return c[k].value();
        else return k == 0 ? c.value() : 0u;
    };
    std::vector<uint32_t> in(current.size() * 4);
    for (size_t i = 0; i < current.size(); ++i)
        for (int k = 0; k < 4; ++k) in[i * 4 + k] = coeff(current[i], k);
    const uint32_t b[4] = {coeff(beta, 0), coeff(beta, 1), coeff(beta, 2), coeff(beta, 3)};
    const size_t n = current.size() / arity;
    DeviceBuffer din(in.size() * 4), dout(n * 16);
    din.upload(in.data(), in.size() * 4);
    check(p3g_fold_matrix_bb4(Context::get().handle(), din.get(), uint32_t(log_height), uint32_t(log_arity), b,
                              dout.get(), nullptr));
    std::vector<uint32_t> out(n * 4);
    dout.download(out.data(), out.size() * 4);
    std::vector<Challenge> res(n);
    for (size_t i = 0; i < n; ++i) {
        if constexpr (EXT) {
            for (int k = 0; k < 4; ++k) res[i][k] = Val(out[i * 4 + k]);
        } else {
            res[i] = Challenge(out[i * 4]);
        }
    }
    return res;
}

// build_merkle_tree_cuda (merkle_tree_cuda.hpp:358-621): the reference's GPU
// tree build with the same template parameters and arguments, returning the
// reference's MerkleTree<F, F, DIGEST_ELEMS> (leaves moved in, every digest
// layer).  The context takes h_poseidon's constants.  Supported: BabyBear
// WIDTH 16 RATE 8 DIGEST 8, Goldilocks WIDTH 8 RATE 4 DIGEST 4.
template <typename F, size_t WIDTH, size_t RATE, size_t DIGEST_ELEMS, size_t ROUNDS_F, size_t ROUNDS_P, uint64_t D,
          class Mat, class Pos>
p3_merkle_tree::MerkleTree<F, F, DIGEST_ELEMS> build_merkle_tree_cuda(std::vector<Mat> matrices, const Pos& h_poseidon,
                                                                      size_t cap_height) {
    static_assert((sizeof(F) == 4 && WIDTH == 16 && RATE == 8 && DIGEST_ELEMS == 8) ||
                      (sizeof(F) == 8 && WIDTH == 8 && RATE == 4 && DIGEST_ELEMS == 4),
                  "BabyBear 16/8/8 or Goldilocks 8/4/4");
    constexpr size_t E = sizeof(F);
    if (matrices.empty()) throw std::invalid_argument("need at least one matrix");
    Context::get().set_poseidon2(h_poseidon.initial_external_constants, h_poseidon.terminal_external_constants,
                                 h_poseidon.internal_constants, uint32_t(D));
    std::vector<std::unique_ptr<DeviceBuffer>> bufs;
    std::vector<p3g_matrix> descs;
    for (const auto& m : matrices) {
        auto words = to_words(m.values);
        bufs.emplace_back(new DeviceBuffer(std::max<size_t>(words.size(), E)));
        if (!words.empty()) bufs.back()->upload(words.data(), words.size());
        descs.push_back(p3g_matrix{bufs.back()->get(), uint64_t(m.height()), uint32_t(m.width()), 0});
    }
    p3g_ctx* ctx = Context::get().handle();
    p3g_tree* tree = nullptr;
    check(p3g_mmcs_commit(ctx, field_id<F>(), descs.data(), descs.size(), uint32_t(cap_height), &tree, nullptr,
                          nullptr));
    p3_merkle_tree::MerkleTree<F, F, DIGEST_ELEMS> out;
    out.digest_layers = download_layers<std::array<F, DIGEST_ELEMS>>(ctx, tree);
    check(p3g_tree_free(ctx, tree, nullptr));
    out.leaves = std::move(matrices);
    return out;
}

// fold_matrix_cuda (fri_fold_cuda.hpp:300-348): the reference's GPU fold, same
// arguments in its order (beta first), host vectors in and out.
template <class Val, class Challenge>
std::vector<Challenge> fold_matrix_cuda(const Challenge& beta, size_t log_arity, size_t log_height,
                                        const std::vector<Challenge>& current) {
    return gpu_fold_matrix<Val, Challenge>(log_height, log_arity, beta, current);
}

// fold_matrix_cuda_device (fri_fold_cuda.hpp:250-277): device buffers already
// sized (d_input n * 2^log_arity values, d_output n), no allocation or copy,
// synchronises the device before returning like the reference.  Challenge is
// BabyBear4 (four canonical u32 coefficients in memory, as the kernel reads them).
template <class Val, class Challenge>
void fold_matrix_cuda_device(const Challenge* d_input, Challenge* d_output, const Challenge& beta, size_t log_arity,
                             size_t log_height, size_t n) {
    static_assert(sizeof(Val) == 4 && sizeof(Challenge) == 16, "fold runs over BabyBear^4");
    if (log_arity < 1 || log_arity > 3) throw std::invalid_argument("log_arity must be 1, 2, or 3");
    if (log_height < log_arity || n != (size_t(1) << log_height) >> log_arity)
        throw std::invalid_argument("fold_matrix_cuda_device: n must be 2^log_height / 2^log_arity");
    const uint32_t b[4] = {beta[0].value(), beta[1].value(), beta[2].value(), beta[3].value()};
    check(p3g_fold_matrix_bb4(Context::get().handle(), d_input, uint32_t(log_height), uint32_t(log_arity), b, d_output,
                              nullptr));
    check(p3g_stream_synchronize(Context::get().handle(), nullptr));
}

// ----------------------------------------------------------------- challenger
// DuplexChallenger<F, Perm, WIDTH, RATE> (duplex_challenger.hpp:42-285) whose
// proof-of-work search, grind (:234-251), runs on the GPU (p3g_grind).  The
// reference keeps its sponge state private, so this class carries its own:
// the same transcript steps -- observations fill an input buffer that is
// written over the first RATE state words when full or before a sample, the
// state is permuted by Perm on the host and its first RATE words become the
// output buffer, sampled from the back.  It has the reference's public
// members and stands in for it wherever a challenger is a template argument,
// e.g. as the inner challenger of a prove_fri transcript.  BabyBear WIDTH 16
// RATE 8 or Goldilocks WIDTH 8 RATE 4; the context's Poseidon2 constants for
// the field (Context::set_poseidon2) must describe the same permutation as Perm.
template <class F, class Perm, size_t WIDTH, size_t RATE>
class GpuDuplexChallenger {
    static_assert((sizeof(F) == 4 && WIDTH == 16 && RATE == 8) || (sizeof(F) == 8 && WIDTH == 8 && RATE == 4),
                  "BabyBear width 16 rate 8, or Goldilocks width 8 rate 4");
    using Word = std::conditional_t<sizeof(F) == 4, uint32_t, uint64_t>;

public:
    static constexpr size_t FIELD_BITS = sizeof(F) == 4 ? 31 : 64;

    explicit GpuDuplexChallenger(Perm perm) : perm_(std::move(perm)), state_{} { in_.reserve(RATE); }

    void observe(F v) {
        out_.clear();
        absorb(v);
    }
    void observe_slice(const std::vector<F>& vs) {
        if (vs.empty()) return;
        out_.clear();
        for (const F& v : vs) absorb(v);
    }
    F sample() {
        if (!in_.empty() || out_.empty()) duplexing();
        F v = out_.back();
        out_.pop_back();
        return v;
    }
    size_t sample_bits(size_t bits) {
        size_t result = 0, left = bits;
        while (left > 0) {
            const uint64_t v = canonical(sample());
            const size_t chunk = left < FIELD_BITS ? left : FIELD_BITS;
            const uint64_t mask = chunk == 64 ? ~uint64_t(0) : (uint64_t(1) << chunk) - 1;
            result |= size_t(v & mask) << (bits - left);
            left -= chunk;
        }
        return result;
    }
    template <class EF>
    EF sample_algebra_element() {
        EF r{};
        for (size_t i = 0; i < EF::DEGREE; ++i) r.coeffs[i] = sample();
        return r;
    }
    template <class EF>
    void observe_algebra_element(const EF& v) {
        out_.clear();
        for (size_t i = 0; i < EF::DEGREE; ++i) absorb(v.coeffs[i]);
    }
    template <class EF>
    void observe_algebra_slice(const std::vector<EF>& vs) {
        if (vs.empty()) return;
        out_.clear();
        for (const EF& v : vs)
            for (size_t i = 0; i < EF::DEGREE; ++i) absorb(v.coeffs[i]);
    }
    template <class Hash>
    void observe_merkle_cap(const std::vector<Hash>& cap) {
        if (cap.empty()) return;
        out_.clear();
        for (const Hash& h : cap)
            for (const F& e : h) absorb(e);
    }

    // The smallest witness whose observation and one sample give an element
    // with `bits` low zero bits; leaves the transcript as the reference's does
    // (witness observed, that sample consumed).
    uint64_t grind(size_t bits) {
        if (bits >= FIELD_BITS) throw std::invalid_argument("grind: PoW bits must be less than FIELD_BITS");
        std::array<Word, WIDTH> st;
        std::array<Word, RATE> in{};
        for (size_t i = 0; i < WIDTH; ++i) st[i] = Word(canonical(state_[i]));
        for (size_t i = 0; i < in_.size(); ++i) in[i] = Word(canonical(in_[i]));
        uint64_t w = 0;
        check(p3g_grind(Context::get().handle(), field_id<F>(), st.data(), in.data(), uint32_t(in_.size()),
                        uint32_t(bits), 0, &w, nullptr));
        observe_witness(w);
        sample();
        return w;
    }
    bool check_witness(size_t bits, uint64_t w) {
        observe_witness(w);
        const uint64_t v = canonical(sample());
        const uint64_t mask = bits >= 64 ? ~uint64_t(0) : (uint64_t(1) << bits) - 1;
        return (v & mask) == 0;
    }

    // The state as p3g_fri_prove takes and returns it (BabyBear), so a device
    // prove_fri can continue this transcript and hand it back.
    p3g_challenger state() const {
        static_assert(sizeof(F) == 4, "p3g_challenger holds the BabyBear challenger");
        p3g_challenger c{};
        for (size_t i = 0; i < WIDTH; ++i) c.sponge_state[i] = uint32_t(canonical(state_[i]));
        for (size_t i = 0; i < in_.size(); ++i) c.input[i] = uint32_t(canonical(in_[i]));
        for (size_t i = 0; i < out_.size(); ++i) c.output[i] = uint32_t(canonical(out_[i]));
        c.n_input = uint32_t(in_.size());
        c.n_output = uint32_t(out_.size());
        return c;
    }
    void set_state(const p3g_challenger& c) {
        static_assert(sizeof(F) == 4, "p3g_challenger holds the BabyBear challenger");
        if (c.n_input >= RATE || c.n_output > RATE) throw std::invalid_argument("set_state: buffers out of range");
        for (size_t i = 0; i < WIDTH; ++i) state_[i] = F(c.sponge_state[i]);
        in_.clear();
        for (uint32_t i = 0; i < c.n_input; ++i) in_.push_back(F(c.input[i]));
        out_.clear();
        for (uint32_t i = 0; i < c.n_output; ++i) out_.push_back(F(c.output[i]));
    }

private:
    void absorb(F v) {
        in_.push_back(v);
        if (in_.size() == RATE) duplexing();
    }
    void observe_witness(uint64_t w) {
        out_.clear();
        absorb(F(uint32_t(w & 0xFFFFFFFFu)));
        absorb(F(uint32_t(w >> 32)));
    }
    void duplexing() {
        std::copy(in_.begin(), in_.end(), state_.begin());
        in_.clear();
        perm_.permute_mut(state_);
        out_.assign(state_.begin(), state_.begin() + RATE);
    }

    Perm perm_;
    std::array<F, WIDTH> state_;
    std::vector<F> in_, out_;
};

// ----------------------------------------------------------------- prove_fri
namespace detail {
template <class T, class = void>
struct has_state : std::false_type {};
template <class T>
struct has_state<T, std::void_t<decltype(std::declval<T&>().state())>> : std::true_type {};
// The GpuDuplexChallenger behind a transcript: the challenger itself, or the
// `inner` challenger of a wrapper (as the FRI tests' transcript holds it).
template <class Challenger>
auto& gpu_challenger(Challenger& c) {
    if constexpr (has_state<Challenger>::value) return c;
    else return c.inner;
}
}  // namespace detail

// prove_fri (fri_prover.hpp:35-265) with the reference's signature, every data
// step and the Fiat-Shamir transcript on the GPU (p3g_fri_prove, one call):
// BabyBear / BabyBear^4, the commit phase's flat MMCS over the context's
// Poseidon2-16, arities 2 to 8.  The challenger is a GpuDuplexChallenger, or a
// wrapper whose `inner` member is one, with the transcript calls of the FRI
// tests' wrapper (fri_test.cpp:100-120); it comes back advanced exactly as the
// reference's prove_fri leaves it.  The input openings are the input MMCS's own
// (input_mmcs.open at each query index, on the host).  Returns the reference's
// FriProof.
template <typename Val, typename Challenge, typename FriMmcs, typename Challenger, typename Witness,
          typename InputMmcs, typename InputProof>
p3_fri::FriProof<Challenge, FriMmcs, Witness, InputProof> gpu_prove_fri(
    const p3_fri::FriParameters<FriMmcs>& params, std::vector<std::vector<Challenge>> inputs, Challenger& challenger,
    const std::vector<typename InputMmcs::ProverData>& input_data, const InputMmcs& input_mmcs) {
    static_assert(sizeof(Val) == 4 && sizeof(Challenge) == 16, "FRI over BabyBear^4");
    using Proof = p3_fri::FriProof<Challenge, FriMmcs, Witness, InputProof>;
    if (inputs.empty()) throw std::invalid_argument("prove_fri: no input vectors");
    auto& ch = detail::gpu_challenger(challenger);
    p3g_fri_params fp{uint32_t(params.log_blowup), uint32_t(params.log_final_poly_len), uint32_t(params.max_log_arity),
                      uint32_t(params.num_queries), uint32_t(params.commit_proof_of_work_bits),
                      uint32_t(params.query_proof_of_work_bits)};
    std::vector<uint32_t> log_h;
    std::vector<std::unique_ptr<DeviceBuffer>> bufs;
    std::vector<const void*> ptrs;
    for (const auto& v : inputs) {
        log_h.push_back(uint32_t(log2_strict(v.size())));
        std::vector<uint32_t> w(v.size() * 4);
        for (size_t i = 0; i < v.size(); ++i)
            for (int k = 0; k < 4; ++k) w[4 * i + k] = uint32_t(v[i][k].value());
        bufs.emplace_back(new DeviceBuffer(w.size() * 4));
        bufs.back()->upload(w.data(), w.size() * 4);
        ptrs.push_back(bufs.back()->get());
    }
    uint32_t nr = 0, las[32];
    check(p3g_fri_rounds(log_h.data(), uint32_t(log_h.size()), &fp, &nr, las));
    const size_t nq = params.num_queries, fpl = size_t(1) << params.log_final_poly_len;
    size_t row_words = 0, path_words = 0;
    std::vector<uint32_t> heights(nr);
    for (uint32_t r = 0, h = log_h[0]; r < nr; h -= las[r], ++r) {
        heights[r] = h;
        row_words += nq * (size_t(4) << las[r]);
        path_words += nq * (h - las[r]) * 8;
    }
    std::vector<uint32_t> commits(size_t(nr) * 8), final_poly(fpl * 4), rows(std::max<size_t>(row_words, 1)),
        paths(std::max<size_t>(path_words, 1));
    std::vector<uint64_t> wits(std::max<uint32_t>(nr, 1)), qidx(std::max<size_t>(nq, 1));
    uint64_t qwit = 0;
    p3g_challenger st = ch.state();
    check(p3g_fri_prove(Context::get().handle(), ptrs.data(), log_h.data(), uint32_t(log_h.size()), &fp, &st,
                        commits.data(), wits.data(), final_poly.data(), &qwit, qidx.data(), rows.data(), paths.data(),
                        nullptr));
    ch.set_state(st);

    auto ext = [](const uint32_t* w) {
        Challenge c{};
        for (int k = 0; k < 4; ++k) c[k] = Val(w[k]);
        return c;
    };
    Proof proof;
    using Commitment = typename decltype(proof.commit_phase_commits)::value_type;
    using Digest = typename Commitment::value_type;
    auto digest = [](const uint32_t* w) {
        Digest d{};
        for (size_t k = 0; k < d.size(); ++k) d[k] = Val(w[k]);
        return d;
    };
    for (uint32_t r = 0; r < nr; ++r) {
        Commitment c;
        c.push_back(digest(&commits[8 * r]));
        proof.commit_phase_commits.push_back(std::move(c));
        proof.commit_pow_witnesses.push_back(Witness(wits[r]));
    }
    for (size_t k = 0; k < fpl; ++k) proof.final_poly.push_back(ext(&final_poly[4 * k]));
    proof.query_pow_witness = Witness(qwit);
    using QP = typename decltype(proof.query_proofs)::value_type;
    for (size_t q = 0; q < nq; ++q) {
        QP qp;
        input_mmcs.open(size_t(qidx[q]), input_data, qp.input_proof);
        size_t ro = 0, po = 0, cur = size_t(qidx[q]);
        for (uint32_t r = 0; r < nr; ++r) {
            const size_t arity = size_t(1) << las[r], depth = heights[r] - las[r];
            typename decltype(qp.commit_phase_openings)::value_type step;
            step.log_arity = uint8_t(las[r]);
            const uint32_t* row = &rows[ro + q * 4 * arity];
            for (size_t j = 0; j < arity; ++j)
                if (j != (cur & (arity - 1))) step.sibling_values.push_back(ext(row + 4 * j));
            const uint32_t* path = &paths[po + q * depth * 8];
            for (size_t l = 0; l < depth; ++l) step.opening_proof.push_back(digest(path + 8 * l));
            qp.commit_phase_openings.push_back(std::move(step));
            ro += nq * 4 * arity;
            po += nq * depth * 8;
            cur >>= las[r];
        }
        proof.query_proofs.push_back(std::move(qp));
    }
    return proof;
}

}  // namespace p3g
