/*
 * oracle.h -- CPU restatement of the reference's trace-commitment path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA
 * path is compared against (and the timed CPU baseline in bench.py).  It is
 * never linked into, loaded by, or called from the product library.
 *
 * Every function restates one reference routine (dloghin/plonky3-gpu,
 * header-only C++ under src/include/) and cites the file:line it follows.
 * Arithmetic is kept in the reference's own representation: canonical
 * BabyBear values in [0, p) with products reduced by `% p`
 * (baby_bear.hpp:75-88), canonical Goldilocks values (goldilocks.hpp:53-100),
 * and BabyBear^4 = BabyBear[x]/(x^4 - 11) (extension_field.hpp:106-131).
 */
#ifndef P3G_ORACLE_H
#define P3G_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_BB_P 0x78000001u
#define ORC_GL_P 0xFFFFFFFF00000001ull

/* ---------------- fields ---------------- */
uint32_t orc_bb_add(uint32_t a, uint32_t b);
uint32_t orc_bb_sub(uint32_t a, uint32_t b);
uint32_t orc_bb_mul(uint32_t a, uint32_t b);
uint32_t orc_bb_pow(uint32_t a, uint64_t e);
uint32_t orc_bb_inv(uint32_t a);
uint32_t orc_bb_two_adic_generator(unsigned bits);

uint64_t orc_gl_add(uint64_t a, uint64_t b);
uint64_t orc_gl_sub(uint64_t a, uint64_t b);
uint64_t orc_gl_mul(uint64_t a, uint64_t b);
uint64_t orc_gl_pow(uint64_t a, uint64_t e);
uint64_t orc_gl_inv(uint64_t a);
uint64_t orc_gl_two_adic_generator(unsigned bits);

void orc_bb4_mul(const uint32_t a[4], const uint32_t b[4], uint32_t out[4]);
void orc_bb4_inv(const uint32_t a[4], uint32_t out[4]);
uint32_t orc_bb4_dth_root(void);

/* ---------------- seeded generators (std::mt19937 / std::mt19937_64) ---- */
void orc_mt19937(uint32_t seed, uint32_t *out, size_t n);
void orc_mt19937_64(uint64_t seed, uint64_t *out, size_t n);

/* ---------------- DFT / LDE ---------------- */
void orc_bb_dft_batch(uint32_t *mat, unsigned log_h, size_t w);
void orc_bb_idft_batch(uint32_t *mat, unsigned log_h, size_t w);
void orc_bb_coset_dft_batch(uint32_t *mat, unsigned log_h, size_t w, uint32_t shift);
void orc_bb_coset_idft_batch(uint32_t *mat, unsigned log_h, size_t w, uint32_t shift);
void orc_bb_reverse_rows(uint32_t *mat, unsigned log_h, size_t w);
/* out has (h << log_blowup) * w elements; nthreads >= 1 splits columns. */
int orc_bb_coset_lde(const uint32_t *in, unsigned log_h, size_t w, unsigned log_blowup,
                     uint32_t shift, int bitrev_out, uint32_t *out, int nthreads);

void orc_gl_dft_batch(uint64_t *mat, unsigned log_h, size_t w);
void orc_gl_idft_batch(uint64_t *mat, unsigned log_h, size_t w);
void orc_gl_coset_dft_batch(uint64_t *mat, unsigned log_h, size_t w, uint64_t shift);
void orc_gl_reverse_rows(uint64_t *mat, unsigned log_h, size_t w);
int orc_gl_coset_lde(const uint64_t *in, unsigned log_h, size_t w, unsigned log_blowup,
                     uint64_t shift, int bitrev_out, uint64_t *out, int nthreads);

/* ---------------- Poseidon2 ---------------- */
#define ORC_P2_MAX_HALF_F 8
#define ORC_P2_MAX_P 32
#define ORC_P2_MAX_W 24
typedef struct {
    int32_t field;      /* 0 = BabyBear, 1 = Goldilocks */
    int32_t width;      /* 8, 12, 16, 20 or 24 */
    int32_t rounds_f;   /* full rounds, even */
    int32_t rounds_p;   /* partial rounds */
    int32_t degree;     /* S-box exponent: 3, 5 or 7 */
    int32_t rate;       /* sponge rate (elements absorbed per permutation) */
    int32_t digest;     /* digest elements (= compression chunk) */
    int32_t pad_;
    uint64_t initial_rc[ORC_P2_MAX_HALF_F * ORC_P2_MAX_W];  /* [rounds_f/2][width] */
    uint64_t terminal_rc[ORC_P2_MAX_HALF_F * ORC_P2_MAX_W]; /* [rounds_f/2][width] */
    uint64_t internal_rc[ORC_P2_MAX_P];                     /* [rounds_p] */
} orc_p2;

void orc_p2_permute_bb(const orc_p2 *p, uint32_t *state);
void orc_p2_permute_gl(const orc_p2 *p, uint64_t *state);
/* DuplexChallenger<F, Perm, width, rate>::grind from the challenger's sponge
 * state (width elements) and n_input < rate pending inputs (u32 BabyBear, u64
 * Goldilocks): the smallest witness below limit, or -1 if none. */
int orc_grind(const orc_p2 *p, const void *state, const void *input, unsigned n_input, unsigned bits,
              uint64_t limit, uint64_t *witness_out);
/* PaddingFreeSponge::hash_iter: elements are u32 (BB) or u64 (GL). */
void orc_p2_hash(const orc_p2 *p, const void *data, size_t len, void *digest_out);
/* TruncatedPermutation<.., 2, digest, width>::compress */
void orc_p2_compress(const orc_p2 *p, const void *left, const void *right, void *out);

/* ---------------- Merkle / MMCS ---------------- */
/* Mixed-height MerkleTreeMmcs::commit (merkle_tree.hpp:84-185).  mats[i] is a
 * row-major height[i] x width[i] matrix (u32 for BB, u64 for GL).  Writes all
 * digest layers bottom-up, concatenated, into layers_out (capacity in digests)
 * and the number of digests per layer into layer_sizes (capacity max_layers).
 * Returns the number of layers, or -1 on bad input. */
int orc_mmcs_commit(const orc_p2 *p, const void *const *mats, const size_t *heights,
                    const size_t *widths, size_t n, unsigned cap_height,
                    void *layers_out, size_t layers_cap, size_t *layer_sizes,
                    size_t max_layers, int nthreads);

/* Flat p3_merkle::MerkleTreeMmcs::commit_matrix (fri_merkle_tree_mmcs.hpp:55-102).
 * Same output convention as orc_mmcs_commit. */
int orc_commit_matrix(const orc_p2 *p, const void *flat, size_t height, size_t width,
                      void *layers_out, size_t layers_cap, size_t *layer_sizes,
                      size_t max_layers, int nthreads);

/* ---------------- FRI ---------------- */
/* TwoAdicFriFolding<BabyBear, BabyBear4>::fold_matrix (fri_folding.hpp:200-222).
 * in: 2^log_height BB4 elements (4 u32 each), out: 2^(log_height-log_arity). */
int orc_fold_matrix_bb4(const uint32_t *in, unsigned log_height, unsigned log_arity,
                        const uint32_t beta[4], uint32_t *out, int nthreads);

/* ---------------- PCS open ---------------- */
/* Opened values of one LDE matrix at point z, as TwoAdicFriPcs::open computes
 * them (two_adic_fri_pcs.hpp:296-335) with compute_diff_invs and
 * interpolate_coset_with_precomputation (interpolation.hpp:93-180):
 *   f(z) = (z^n - g^n) * sum_i d_i * f_i / (z - g h_i),  d_i = h_i / (n g^(n-1)),
 * h_i = omega_n^i; lde: n x w canonical, natural row order; out: w BB4. */
void orc_pcs_open_values(const uint32_t *lde, unsigned log_n, size_t w, uint32_t shift,
                         const uint32_t z[4], uint32_t *out, int nthreads);
/* The reduced-opening accumulation of one matrix (two_adic_fri_pcs.hpp:350-410):
 *   q[k] += sum_p sum_c alpha^(ap0 + p*w + c) * (opened[p][c] - lde[k][c]) / (z_p - g omega_n^k)
 * for k < n (natural order), m points z (m x 4), opened m x w BB4. */
void orc_pcs_reduce(const uint32_t *lde, unsigned log_n, size_t w, uint32_t shift,
                    const uint32_t *z, size_t m, const uint32_t *opened, const uint32_t alpha[4],
                    uint64_t ap0, uint32_t *q, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
