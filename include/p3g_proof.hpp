// p3g_proof.hpp -- a byte format for the prover's outputs: FRI proofs, PCS
// opened values and Merkle caps.
//
// The reference defines the proof objects (fri_proof.hpp:10-32, merkle_cap.hpp,
// two_adic_fri_pcs.hpp:88-92) but no wire format.  This header gives one, so a
// proof built with the GPU adapters (or the reference alone) can leave the
// process and be read back into the same C++ types for the reference's
// verifier.  Header-only C++17, no dependency on the reference's headers: the
// objects are recognised by their members.
//
//   std::vector<uint8_t> bytes = p3g::wire::encode(proof);
//   auto back = p3g::wire::decode<decltype(proof)>(bytes.data(), bytes.size());
//
// Layout, little-endian:
//   header        "P3GW", u32 version (1)
//   base field    BabyBear u32 / Goldilocks u64, canonical (decode rejects
//                 non-canonical values)
//   extension     its coefficients in order (a type with `coeffs`)
//   std::vector   u32 length, then the elements
//   std::array    the elements
//   integers      u8 / u32 / u64 as declared (size_t as u64)
//   FriProof      commit_phase_commits, commit_pow_witnesses, query_proofs,
//                 final_poly, query_pow_witness
//   QueryProof    input_proof, commit_phase_openings
//   CommitPhaseProofStep  log_arity (u8), sibling_values, opening_proof
//   row opening   row_index, row_values (PcsQueryInputMmcs::OpeningProof)
// Truncated or malformed input raises std::invalid_argument.
#pragma once

#include <array>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <type_traits>
#include <utility>
#include <vector>

namespace p3g {
namespace wire {

constexpr uint32_t VERSION = 1;

struct Writer {
    std::vector<uint8_t> buf;
    template <class U>
    void raw(U v) {
        static_assert(std::is_integral<U>::value, "integers only");
        for (size_t i = 0; i < sizeof(U); ++i) buf.push_back(uint8_t(uint64_t(v) >> (8 * i)));
    }
};

struct Reader {
    const uint8_t* p;
    size_t n, off = 0;
    template <class U>
    U raw() {
        if (n - off < sizeof(U)) throw std::invalid_argument("p3g wire: truncated input");
        uint64_t v = 0;
        for (size_t i = 0; i < sizeof(U); ++i) v |= uint64_t(p[off + i]) << (8 * i);
        off += sizeof(U);
        return U(v);
    }
};

// ---------------------------------------------------------------- detection
template <class T, class = void>
struct is_vector : std::false_type {};
template <class E, class A>
struct is_vector<std::vector<E, A>> : std::true_type {};
template <class T>
struct is_array : std::false_type {};
template <class E, size_t N>
struct is_array<std::array<E, N>> : std::true_type {};

#define P3G_WIRE_HAS(name, expr)                                                 \
    template <class T, class = void>                                             \
    struct name : std::false_type {};                                            \
    template <class T>                                                           \
    struct name<T, std::void_t<decltype(expr)>> : std::true_type {};
P3G_WIRE_HAS(has_value, std::declval<const T&>().value())
P3G_WIRE_HAS(has_canonical, std::declval<const T&>().as_canonical_u64())
P3G_WIRE_HAS(has_coeffs, std::declval<const T&>().coeffs)
P3G_WIRE_HAS(is_fri_proof, std::declval<const T&>().commit_phase_commits)
P3G_WIRE_HAS(is_query_proof, std::declval<const T&>().commit_phase_openings)
P3G_WIRE_HAS(is_step, std::declval<const T&>().sibling_values)
P3G_WIRE_HAS(is_row_opening, std::declval<const T&>().row_values)
#undef P3G_WIRE_HAS

// A base field element: BabyBear (4 bytes, value()) or Goldilocks (8 bytes,
// as_canonical_u64()).
template <class T>
constexpr bool is_base_field() {
    return !std::is_arithmetic<T>::value && !has_coeffs<T>::value &&
           ((sizeof(T) == 4 && has_value<T>::value) || (sizeof(T) == 8 && has_canonical<T>::value));
}

template <class T>
void put(Writer& w, const T& x);
template <class T>
void get(Reader& r, T& x);

template <class T>
void put(Writer& w, const T& x) {
    if constexpr (std::is_same<T, bool>::value) {
        w.raw<uint8_t>(x ? 1 : 0);
    } else if constexpr (std::is_same<T, size_t>::value) {
        w.raw<uint64_t>(uint64_t(x));
    } else if constexpr (std::is_integral<T>::value) {
        w.raw<T>(x);
    } else if constexpr (is_base_field<T>()) {
        if constexpr (sizeof(T) == 4) w.raw<uint32_t>(uint32_t(x.value()));
        else w.raw<uint64_t>(x.as_canonical_u64());
    } else if constexpr (has_coeffs<T>::value) {
        for (const auto& c : x.coeffs) put(w, c);
    } else if constexpr (is_vector<T>::value) {
        if (x.size() > 0xFFFFFFFFull) throw std::invalid_argument("p3g wire: vector too long");
        w.raw<uint32_t>(uint32_t(x.size()));
        for (const auto& e : x) put(w, e);
    } else if constexpr (is_array<T>::value) {
        for (const auto& e : x) put(w, e);
    } else if constexpr (is_fri_proof<T>::value) {
        put(w, x.commit_phase_commits);
        put(w, x.commit_pow_witnesses);
        put(w, x.query_proofs);
        put(w, x.final_poly);
        put(w, x.query_pow_witness);
    } else if constexpr (is_query_proof<T>::value) {
        put(w, x.input_proof);
        put(w, x.commit_phase_openings);
    } else if constexpr (is_step<T>::value) {
        put(w, x.log_arity);
        put(w, x.sibling_values);
        put(w, x.opening_proof);
    } else if constexpr (is_row_opening<T>::value) {
        put(w, x.row_index);
        put(w, x.row_values);
    } else {
        static_assert(sizeof(T) == 0, "p3g wire: no encoding for this type");
    }
}

template <class T>
void get(Reader& r, T& x) {
    if constexpr (std::is_same<T, bool>::value) {
        x = r.raw<uint8_t>() != 0;
    } else if constexpr (std::is_same<T, size_t>::value) {
        x = size_t(r.raw<uint64_t>());
    } else if constexpr (std::is_integral<T>::value) {
        x = r.raw<T>();
    } else if constexpr (is_base_field<T>()) {
        if constexpr (sizeof(T) == 4) {
            const uint32_t v = r.raw<uint32_t>();
            x = T(v);
            if (uint32_t(x.value()) != v) throw std::invalid_argument("p3g wire: non-canonical field element");
        } else {
            const uint64_t v = r.raw<uint64_t>();
            x = T(v);
            if (x.as_canonical_u64() != v) throw std::invalid_argument("p3g wire: non-canonical field element");
        }
    } else if constexpr (has_coeffs<T>::value) {
        for (auto& c : x.coeffs) get(r, c);
    } else if constexpr (is_vector<T>::value) {
        const uint32_t n = r.raw<uint32_t>();
        if (n > r.n - r.off) throw std::invalid_argument("p3g wire: length beyond the input");  // >= 1 byte each
        x.clear();
        x.resize(n);
        for (auto& e : x) get(r, e);
    } else if constexpr (is_array<T>::value) {
        for (auto& e : x) get(r, e);
    } else if constexpr (is_fri_proof<T>::value) {
        get(r, x.commit_phase_commits);
        get(r, x.commit_pow_witnesses);
        get(r, x.query_proofs);
        get(r, x.final_poly);
        get(r, x.query_pow_witness);
    } else if constexpr (is_query_proof<T>::value) {
        get(r, x.input_proof);
        get(r, x.commit_phase_openings);
    } else if constexpr (is_step<T>::value) {
        get(r, x.log_arity);
        get(r, x.sibling_values);
        get(r, x.opening_proof);
    } else if constexpr (is_row_opening<T>::value) {
        get(r, x.row_index);
        get(r, x.row_values);
    } else {
        static_assert(sizeof(T) == 0, "p3g wire: no decoding for this type");
    }
}

template <class T>
std::vector<uint8_t> encode(const T& obj) {
    Writer w;
    for (char c : {'P', '3', 'G', 'W'}) w.raw<uint8_t>(uint8_t(c));
    w.raw<uint32_t>(VERSION);
    put(w, obj);
    return std::move(w.buf);
}

template <class T>
T decode(const uint8_t* data, size_t n) {
    Reader r{data, n};
    for (char c : {'P', '3', 'G', 'W'})
        if (r.raw<uint8_t>() != uint8_t(c)) throw std::invalid_argument("p3g wire: not a p3g proof");
    if (r.raw<uint32_t>() != VERSION) throw std::invalid_argument("p3g wire: unknown version");
    T obj{};
    get(r, obj);
    if (r.off != n) throw std::invalid_argument("p3g wire: trailing bytes");
    return obj;
}

}  // namespace wire
}  // namespace p3g
