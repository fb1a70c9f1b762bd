/*
 * oracle.c -- CPU restatement of the reference's trace-commitment path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
 * baseline.  Nothing in the product library links or calls this file.
 *
 * Each routine restates the reference (dloghin/plonky3-gpu, src/include/...)
 * with the same operation order and the same arithmetic representation, so
 * that its cost is representative when timed as the CPU baseline.  The
 * optional `nthreads` argument splits independent work (columns of an LDE,
 * rows of a leaf layer, outputs of a fold) across POSIX threads; the
 * arithmetic per element is unchanged.
 */
#include "oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

/* ======================================================================
 * Parallel helper
 * ====================================================================== */
typedef void (*orc_range_fn)(void *ctx, size_t lo, size_t hi);
typedef struct {
    orc_range_fn fn;
    void *ctx;
    size_t lo, hi;
} orc_job;

static void *orc_job_run(void *arg) {
    orc_job *j = (orc_job *)arg;
    j->fn(j->ctx, j->lo, j->hi);
    return NULL;
}

static void orc_parallel(size_t n, int nthreads, orc_range_fn fn, void *ctx) {
    if (nthreads <= 1 || n < 2) {
        fn(ctx, 0, n);
        return;
    }
    if ((size_t)nthreads > n) nthreads = (int)n;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    orc_job *jobs = (orc_job *)malloc(sizeof(orc_job) * (size_t)nthreads);
    size_t chunk = (n + (size_t)nthreads - 1) / (size_t)nthreads;
    int started = 0;
    for (int t = 0; t < nthreads; ++t) {
        size_t lo = (size_t)t * chunk, hi = lo + chunk;
        if (lo >= n) break;
        if (hi > n) hi = n;
        jobs[t].fn = fn; jobs[t].ctx = ctx; jobs[t].lo = lo; jobs[t].hi = hi;
        if (t == 0) continue; /* run on the calling thread below */
        pthread_create(&th[t], NULL, orc_job_run, &jobs[t]);
        started = t;
    }
    orc_job_run(&jobs[0]);
    for (int t = 1; t <= started; ++t) pthread_join(th[t], NULL);
    free(th);
    free(jobs);
}

static size_t orc_rev_bits(size_t x, unsigned bits) {
    /* p3_util/util.hpp:38-47 */
    size_t r = 0;
    for (unsigned i = 0; i < bits; ++i) {
        r = (r << 1) | (x & 1);
        x >>= 1;
    }
    return r;
}

/* ======================================================================
 * BabyBear: canonical u32, products reduced by % p (baby_bear.hpp:75-105)
 * ====================================================================== */
uint32_t orc_bb_add(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a + b) % ORC_BB_P); }
uint32_t orc_bb_sub(uint32_t a, uint32_t b) {
    return (uint32_t)(((uint64_t)a + ORC_BB_P - b) % ORC_BB_P);
}
uint32_t orc_bb_mul(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) % ORC_BB_P); }

uint32_t orc_bb_pow(uint32_t a, uint64_t e) {
    /* field.hpp:84-101 square-and-multiply */
    uint32_t r = 1, b = a;
    while (e) {
        if (e & 1) r = orc_bb_mul(r, b);
        b = orc_bb_mul(b, b);
        e >>= 1;
    }
    return r;
}
uint32_t orc_bb_inv(uint32_t a) { return orc_bb_pow(a, ORC_BB_P - 2); } /* baby_bear.hpp:95-105 */

uint32_t orc_bb_two_adic_generator(unsigned bits) {
    /* baby_bear.hpp:131-145: 440564289^(2^(27-bits)) */
    if (bits > 27) return 0;
    return orc_bb_pow(440564289u, (uint64_t)1 << (27 - bits));
}

/* ======================================================================
 * Goldilocks: canonical u64 (goldilocks.hpp:53-117)
 * ====================================================================== */
uint64_t orc_gl_add(uint64_t a, uint64_t b) { return (uint64_t)(((u128)a + b) % ORC_GL_P); }
uint64_t orc_gl_sub(uint64_t a, uint64_t b) {
    return (uint64_t)(((u128)a + ORC_GL_P - (b % ORC_GL_P)) % ORC_GL_P);
}
uint64_t orc_gl_mul(uint64_t a, uint64_t b) { return (uint64_t)(((u128)a * b) % ORC_GL_P); }
uint64_t orc_gl_pow(uint64_t a, uint64_t e) {
    uint64_t r = 1, b = a % ORC_GL_P;
    while (e) {
        if (e & 1) r = orc_gl_mul(r, b);
        b = orc_gl_mul(b, b);
        e >>= 1;
    }
    return r;
}
uint64_t orc_gl_inv(uint64_t a) { return orc_gl_pow(a, ORC_GL_P - 2); }
uint64_t orc_gl_two_adic_generator(unsigned bits) {
    /* goldilocks.hpp has no two-adic generator; the standard one is
     * 7^((p-1)/2^bits) with 7 the multiplicative generator (two-adicity 32). */
    if (bits > 32) return 0;
    return orc_gl_pow(7, (ORC_GL_P - 1) >> bits);
}

/* ======================================================================
 * BabyBear^4 = BabyBear[x]/(x^4 - 11)  (extension_field.hpp:106-131, 396-446)
 * ====================================================================== */
void orc_bb4_mul(const uint32_t a[4], const uint32_t b[4], uint32_t out[4]) {
    uint32_t r[4] = {0, 0, 0, 0};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            uint32_t prod = orc_bb_mul(a[i], b[j]);
            int idx = i + j;
            if (idx < 4) r[idx] = orc_bb_add(r[idx], prod);
            else r[idx - 4] = orc_bb_add(r[idx - 4], orc_bb_mul(prod, 11));
        }
    memcpy(out, r, sizeof(r));
}

uint32_t orc_bb4_dth_root(void) { return orc_bb_pow(11, (ORC_BB_P - 1) / 4); }

void orc_bb4_inv(const uint32_t a[4], uint32_t out[4]) {
    /* Frobenius/norm inverse, extension_field.hpp:396-446 */
    uint32_t z = orc_bb4_dth_root();
    uint32_t z2 = orc_bb_mul(z, z), z3 = orc_bb_mul(z2, z);
    uint32_t pa[4] = {a[0], orc_bb_mul(a[1], z), orc_bb_mul(a[2], z2), orc_bb_mul(a[3], z3)};
    uint32_t p2a[4] = {a[0], orc_bb_mul(a[1], z2), a[2], orc_bb_mul(a[3], z2)};
    uint32_t p3a[4] = {a[0], orc_bb_mul(a[1], z3), orc_bb_mul(a[2], z2), orc_bb_mul(a[3], z)};
    uint32_t a_pa[4], p23[4], norm[4], num[4];
    orc_bb4_mul(a, pa, a_pa);
    orc_bb4_mul(p2a, p3a, p23);
    orc_bb4_mul(a_pa, p23, norm);
    uint32_t ninv = orc_bb_inv(norm[0]);
    orc_bb4_mul(pa, p23, num);
    for (int i = 0; i < 4; ++i) out[i] = orc_bb_mul(num[i], ninv);
}

static int bb4_eq(const uint32_t a[4], const uint32_t b[4]) {
    return a[0] == b[0] && a[1] == b[1] && a[2] == b[2] && a[3] == b[3];
}
static void bb4_sub(const uint32_t a[4], const uint32_t b[4], uint32_t out[4]) {
    for (int i = 0; i < 4; ++i) out[i] = orc_bb_sub(a[i], b[i]);
}
static void bb4_embed(uint32_t v, uint32_t out[4]) {
    out[0] = v; out[1] = 0; out[2] = 0; out[3] = 0;
}

/* ======================================================================
 * MT19937 / MT19937-64 (the published Matsumoto-Nishimura generators, as
 * std::mt19937 and std::mt19937_64 define them)
 * ====================================================================== */
void orc_mt19937(uint32_t seed, uint32_t *out, size_t n) {
    uint32_t mt[624];
    int idx = 624;
    mt[0] = seed;
    for (int i = 1; i < 624; ++i) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
    for (size_t k = 0; k < n; ++k) {
        if (idx >= 624) {
            for (int i = 0; i < 624; ++i) {
                uint32_t y = (mt[i] & 0x80000000u) | (mt[(i + 1) % 624] & 0x7fffffffu);
                mt[i] = mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
            }
            idx = 0;
        }
        uint32_t y = mt[idx++];
        y ^= y >> 11;
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= y >> 18;
        out[k] = y;
    }
}

void orc_mt19937_64(uint64_t seed, uint64_t *out, size_t n) {
    uint64_t mt[312];
    int idx = 312;
    mt[0] = seed;
    for (int i = 1; i < 312; ++i)
        mt[i] = 6364136223846793005ull * (mt[i - 1] ^ (mt[i - 1] >> 62)) + (uint64_t)i;
    for (size_t k = 0; k < n; ++k) {
        if (idx >= 312) {
            for (int i = 0; i < 312; ++i) {
                uint64_t y = (mt[i] & 0xFFFFFFFF80000000ull) | (mt[(i + 1) % 312] & 0x7FFFFFFFull);
                mt[i] = mt[(i + 156) % 312] ^ (y >> 1) ^ ((y & 1ull) ? 0xB5026F5AA96619E9ull : 0ull);
            }
            idx = 0;
        }
        uint64_t x = mt[idx++];
        x ^= (x >> 29) & 0x5555555555555555ull;
        x ^= (x << 17) & 0x71D67FFFEDA60000ull;
        x ^= (x << 37) & 0xFFF7EEE000000000ull;
        x ^= x >> 43;
        out[k] = x;
    }
}

/* ======================================================================
 * Radix2Dit restated on a column range [c0, c1) of a row-major matrix with
 * row stride w (radix2_dit.hpp:46-233, butterflies.hpp, util.hpp:33-45).
 * Columns are independent polynomials, so a column split gives the same
 * result as the reference's whole-row loops.
 * ====================================================================== */
#define DEFINE_DFT(PFX, T, ADD, SUB, MUL, INV, GEN)                                          \
    static void PFX##_swap_rows(T *m, size_t w, size_t c0, size_t c1, size_t i, size_t j) { \
        T *a = m + i * w, *b = m + j * w;                                                    \
        for (size_t c = c0; c < c1; ++c) { T t = a[c]; a[c] = b[c]; b[c] = t; }              \
    }                                                                                        \
    static void PFX##_bitrev_rows(T *m, unsigned log_h, size_t w, size_t c0, size_t c1) {    \
        size_t h = (size_t)1 << log_h;                                                       \
        for (size_t i = 0; i < h; ++i) {                                                     \
            size_t j = orc_rev_bits(i, log_h);                                               \
            if (i < j) PFX##_swap_rows(m, w, c0, c1, i, j);                                  \
        }                                                                                    \
    }                                                                                        \
    static T *PFX##_twiddles(unsigned log_h) {                                               \
        size_t half = ((size_t)1 << log_h) / 2;                                              \
        T *tw = (T *)malloc(sizeof(T) * (half ? half : 1));                                  \
        T root = GEN(log_h), cur = 1;                                                        \
        for (size_t i = 0; i < half; ++i) { tw[i] = cur; cur = MUL(cur, root); }             \
        return tw;                                                                           \
    }                                                                                        \
    static void PFX##_dft_cols(T *m, unsigned log_h, size_t w, size_t c0, size_t c1) {       \
        size_t h = (size_t)1 << log_h;                                                       \
        if (h <= 1) return;                                                                  \
        PFX##_bitrev_rows(m, log_h, w, c0, c1);                                              \
        T *tw = PFX##_twiddles(log_h);                                                       \
        size_t half_n = h / 2;                                                               \
        for (unsigned l = 0; l < log_h; ++l) {                                               \
            size_t half = (size_t)1 << l, step = half * 2, stride = half_n >> l;             \
            for (size_t blk = 0; blk < h; blk += step) {                                     \
                T *a = m + blk * w, *b = m + (blk + half) * w;                               \
                for (size_t c = c0; c < c1; ++c) {                                           \
                    T s = ADD(a[c], b[c]), d = SUB(a[c], b[c]);                              \
                    a[c] = s; b[c] = d;                                                      \
                }                                                                            \
                for (size_t j = 1; j < half; ++j) {                                          \
                    T twd = tw[j * stride];                                                  \
                    T *aj = m + (blk + j) * w, *bj = m + (blk + half + j) * w;               \
                    for (size_t c = c0; c < c1; ++c) {                                       \
                        T ai = aj[c], bi = MUL(twd, bj[c]);                                  \
                        aj[c] = ADD(ai, bi); bj[c] = SUB(ai, bi);                            \
                    }                                                                        \
                }                                                                            \
            }                                                                                \
        }                                                                                    \
        free(tw);                                                                            \
    }                                                                                        \
    static void PFX##_idft_cols(T *m, unsigned log_h, size_t w, size_t c0, size_t c1) {      \
        size_t h = (size_t)1 << log_h;                                                       \
        if (h <= 1) return;                                                                  \
        PFX##_dft_cols(m, log_h, w, c0, c1);                                                 \
        size_t lo = 1, hi = h - 1;                                                           \
        while (lo < hi) { PFX##_swap_rows(m, w, c0, c1, lo, hi); ++lo; --hi; }               \
        T inv_n = 1, inv_two = INV(2);                                                       \
        for (unsigned k = 0; k < log_h; ++k) inv_n = MUL(inv_n, inv_two);                    \
        for (size_t r = 0; r < h; ++r)                                                       \
            for (size_t c = c0; c < c1; ++c) m[r * w + c] = MUL(m[r * w + c], inv_n);        \
    }                                                                                        \
    static void PFX##_coset_dft_cols(T *m, unsigned log_h, size_t w, size_t c0, size_t c1,   \
                                     T shift) {                                              \
        size_t h = (size_t)1 << log_h;                                                       \
        T sp = shift;                                                                        \
        for (size_t i = 1; i < h; ++i) {                                                     \
            for (size_t c = c0; c < c1; ++c) m[i * w + c] = MUL(m[i * w + c], sp);           \
            sp = MUL(sp, shift);                                                             \
        }                                                                                    \
        PFX##_dft_cols(m, log_h, w, c0, c1);                                                 \
    }                                                                                        \
    typedef struct {                                                                         \
        const T *in; T *out; unsigned log_h, log_blowup; size_t w; T shift; int bitrev;      \
    } PFX##_lde_ctx;                                                                         \
    static void PFX##_lde_range(void *vctx, size_t c0, size_t c1) {                          \
        PFX##_lde_ctx *x = (PFX##_lde_ctx *)vctx;                                            \
        size_t h = (size_t)1 << x->log_h, H = h << x->log_blowup, w = x->w;                  \
        for (size_t r = 0; r < h; ++r)                                                       \
            memcpy(x->out + r * w + c0, x->in + r * w + c0, sizeof(T) * (c1 - c0));          \
        PFX##_idft_cols(x->out, x->log_h, w, c0, c1);                                        \
        for (size_t r = h; r < H; ++r) memset(x->out + r * w + c0, 0, sizeof(T) * (c1 - c0)); \
        PFX##_coset_dft_cols(x->out, x->log_h + x->log_blowup, w, c0, c1, x->shift);         \
        if (x->bitrev) PFX##_bitrev_rows(x->out, x->log_h + x->log_blowup, w, c0, c1);       \
    }

DEFINE_DFT(bb, uint32_t, orc_bb_add, orc_bb_sub, orc_bb_mul, orc_bb_inv, orc_bb_two_adic_generator)
DEFINE_DFT(gl, uint64_t, orc_gl_add, orc_gl_sub, orc_gl_mul, orc_gl_inv, orc_gl_two_adic_generator)

void orc_bb_dft_batch(uint32_t *m, unsigned log_h, size_t w) { bb_dft_cols(m, log_h, w, 0, w); }
void orc_bb_idft_batch(uint32_t *m, unsigned log_h, size_t w) { bb_idft_cols(m, log_h, w, 0, w); }
void orc_bb_coset_dft_batch(uint32_t *m, unsigned log_h, size_t w, uint32_t shift) {
    bb_coset_dft_cols(m, log_h, w, 0, w, shift);
}
void orc_bb_coset_idft_batch(uint32_t *m, unsigned log_h, size_t w, uint32_t shift) {
    /* radix2_dit.hpp:194-210 */
    bb_idft_cols(m, log_h, w, 0, w);
    size_t h = (size_t)1 << log_h;
    uint32_t is = orc_bb_inv(shift), ip = is;
    for (size_t i = 1; i < h; ++i) {
        for (size_t c = 0; c < w; ++c) m[i * w + c] = orc_bb_mul(m[i * w + c], ip);
        ip = orc_bb_mul(ip, is);
    }
}
void orc_bb_reverse_rows(uint32_t *m, unsigned log_h, size_t w) { bb_bitrev_rows(m, log_h, w, 0, w); }
void orc_gl_dft_batch(uint64_t *m, unsigned log_h, size_t w) { gl_dft_cols(m, log_h, w, 0, w); }
void orc_gl_idft_batch(uint64_t *m, unsigned log_h, size_t w) { gl_idft_cols(m, log_h, w, 0, w); }
void orc_gl_coset_dft_batch(uint64_t *m, unsigned log_h, size_t w, uint64_t shift) {
    gl_coset_dft_cols(m, log_h, w, 0, w, shift);
}
void orc_gl_reverse_rows(uint64_t *m, unsigned log_h, size_t w) { gl_bitrev_rows(m, log_h, w, 0, w); }

int orc_bb_coset_lde(const uint32_t *in, unsigned log_h, size_t w, unsigned log_blowup,
                     uint32_t shift, int bitrev_out, uint32_t *out, int nthreads) {
    if (log_h + log_blowup > 27) return -1;
    bb_lde_ctx x = {in, out, log_h, log_blowup, w, shift, bitrev_out};
    orc_parallel(w, nthreads, bb_lde_range, &x);
    return 0;
}
int orc_gl_coset_lde(const uint64_t *in, unsigned log_h, size_t w, unsigned log_blowup,
                     uint64_t shift, int bitrev_out, uint64_t *out, int nthreads) {
    if (log_h + log_blowup > 32) return -1;
    gl_lde_ctx x = {in, out, log_h, log_blowup, w, shift, bitrev_out};
    orc_parallel(w, nthreads, gl_lde_range, &x);
    return 0;
}

/* ======================================================================
 * Poseidon2 (poseidon2_cuda.hpp:57-116; external.hpp:67-77, 170-201;
 * generic.hpp:148-175; field.hpp:105-127)
 * ====================================================================== */
#define DEFINE_P2(PFX, T, ADD, MUL)                                                         \
    static T PFX##_sbox(T x, int d) {                                                       \
        if (d == 7) { T sq = MUL(x, x), cu = MUL(sq, x), qu = MUL(sq, sq); return MUL(cu, qu); } \
        if (d == 5) { T sq = MUL(x, x); return MUL(MUL(sq, sq), x); }                       \
        if (d == 3) { return MUL(MUL(x, x), x); }                                           \
        T r = 1;                                                                            \
        for (int i = 0; i < d; ++i) r = MUL(r, x);                                          \
        return r;                                                                           \
    }                                                                                       \
    static void PFX##_mat4(T *x) {                                                          \
        T t01 = ADD(x[0], x[1]), t23 = ADD(x[2], x[3]);                                     \
        T t0123 = ADD(t01, t23);                                                            \
        T t01123 = ADD(t0123, x[1]), t01233 = ADD(t0123, x[3]);                             \
        x[3] = ADD(t01233, ADD(x[0], x[0]));                                                \
        x[1] = ADD(t01123, ADD(x[2], x[2]));                                                \
        x[0] = ADD(t01123, t01);                                                            \
        x[2] = ADD(t01233, t23);                                                            \
    }                                                                                       \
    static void PFX##_mds_light(T *s, int w) {                                              \
        if (w == 2 || w == 3) {                                                             \
            T sum = 0;                                                                      \
            for (int i = 0; i < w; ++i) sum = ADD(sum, s[i]);                               \
            for (int i = 0; i < w; ++i) s[i] = ADD(s[i], sum);                              \
            return;                                                                         \
        }                                                                                   \
        for (int i = 0; i < w; i += 4) PFX##_mat4(s + i);                                   \
        T sums[4];                                                                          \
        for (int k = 0; k < 4; ++k) {                                                       \
            sums[k] = 0;                                                                    \
            for (int j = k; j < w; j += 4) sums[k] = ADD(sums[k], s[j]);                    \
        }                                                                                   \
        for (int i = 0; i < w; ++i) s[i] = ADD(s[i], sums[i % 4]);                          \
    }                                                                                       \
    static void PFX##_internal(T *s, int w) {                                               \
        T sum = 0;                                                                          \
        for (int i = 0; i < w; ++i) sum = ADD(sum, s[i]);                                   \
        T diag = 1;                                                                         \
        for (int i = 0; i < w; ++i) {                                                       \
            s[i] = ADD(MUL(s[i], diag), sum);                                               \
            diag = ADD(diag, diag);                                                         \
        }                                                                                   \
    }                                                                                       \
    static void PFX##_permute(const orc_p2 *p, T *s) {                                      \
        int w = p->width, hf = p->rounds_f / 2;                                             \
        PFX##_mds_light(s, w);                                                              \
        for (int r = 0; r < hf; ++r) {                                                      \
            for (int i = 0; i < w; ++i)                                                     \
                s[i] = PFX##_sbox(ADD(s[i], (T)p->initial_rc[r * w + i]), p->degree);       \
            PFX##_mds_light(s, w);                                                          \
        }                                                                                   \
        for (int r = 0; r < p->rounds_p; ++r) {                                             \
            s[0] = PFX##_sbox(ADD(s[0], (T)p->internal_rc[r]), p->degree);                  \
            PFX##_internal(s, w);                                                           \
        }                                                                                   \
        for (int r = 0; r < hf; ++r) {                                                      \
            for (int i = 0; i < w; ++i)                                                     \
                s[i] = PFX##_sbox(ADD(s[i], (T)p->terminal_rc[r * w + i]), p->degree);      \
            PFX##_mds_light(s, w);                                                          \
        }                                                                                   \
    }

DEFINE_P2(p2bb, uint32_t, orc_bb_add, orc_bb_mul)
DEFINE_P2(p2gl, uint64_t, orc_gl_add, orc_gl_mul)

void orc_p2_permute_bb(const orc_p2 *p, uint32_t *state) { p2bb_permute(p, state); }
void orc_p2_permute_gl(const orc_p2 *p, uint64_t *state) { p2gl_permute(p, state); }

/* DuplexChallenger::grind (duplex_challenger.hpp:234-251), searched in order
 * exactly as the reference does: each candidate replays the challenger's
 * absorb / duplexing / sample steps (:51-73, 115-124) on a copy of the state.
 * The state is held as u64 for both fields. */
typedef struct {
    uint64_t st[ORC_P2_MAX_W];
    uint64_t in[ORC_P2_MAX_W];
    int n_in, n_out;
} orc_chal;

static void chal_duplex(const orc_p2 *p, orc_chal *c) {
    for (int i = 0; i < c->n_in; ++i) c->st[i] = c->in[i];
    c->n_in = 0;
    if (p->field == 0) {
        uint32_t s[ORC_P2_MAX_W];
        for (int i = 0; i < p->width; ++i) s[i] = (uint32_t)c->st[i];
        p2bb_permute(p, s);
        for (int i = 0; i < p->width; ++i) c->st[i] = s[i];
    } else {
        p2gl_permute(p, c->st);
    }
    c->n_out = p->rate;  /* output buffer = st[0..rate), popped from the back */
}

static void chal_absorb(const orc_p2 *p, orc_chal *c, uint64_t v) {
    c->in[c->n_in++] = v;
    if (c->n_in == p->rate) chal_duplex(p, c);
}

int orc_grind(const orc_p2 *p, const void *state, const void *input, unsigned n_input, unsigned bits,
              uint64_t limit, uint64_t *witness_out) {
    if ((int)n_input >= p->rate) return -1;
    const uint64_t mask = bits >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << bits) - 1);
    orc_chal saved;
    memset(&saved, 0, sizeof saved);
    for (int i = 0; i < p->width; ++i)
        saved.st[i] = p->field == 0 ? ((const uint32_t *)state)[i] : ((const uint64_t *)state)[i];
    for (unsigned i = 0; i < n_input; ++i)
        saved.in[i] = p->field == 0 ? ((const uint32_t *)input)[i] : ((const uint64_t *)input)[i];
    saved.n_in = (int)n_input;
    for (uint64_t w = 0; w < limit; ++w) {
        orc_chal a = saved;
        a.n_out = 0;  /* observe_witness clears the output buffer */
        const uint32_t lo = (uint32_t)w, hi = (uint32_t)(w >> 32);
        chal_absorb(p, &a, p->field == 0 ? lo % ORC_BB_P : lo);
        chal_absorb(p, &a, p->field == 0 ? hi % ORC_BB_P : hi);
        if (a.n_in > 0 || a.n_out == 0) chal_duplex(p, &a);
        uint64_t v = a.st[a.n_out - 1];
        if (p->field != 0) v %= ORC_GL_P;
        if ((v & mask) == 0) {
            *witness_out = w;
            return 0;
        }
    }
    return -1;
}

/* A sponge that absorbs from a list of row slices without building a flat
 * copy; identical to hash_iter over the concatenation
 * (padding_free_sponge.hpp:63-113). */
typedef struct {
    const void *ptr;
    size_t len;
} orc_slice;

static void orc_hash_slices(const orc_p2 *p, const orc_slice *sl, size_t nsl, void *digest_out) {
    int W = p->width, RATE = p->rate, OUT = p->digest;
    if (p->field == 0) {
        uint32_t st[ORC_P2_MAX_W] = {0};
        size_t si = 0, pos = 0;
        for (;;) {
            int i = 0;
            while (i < RATE) {
                while (si < nsl && pos >= sl[si].len) { ++si; pos = 0; }
                if (si >= nsl) break;
                st[i++] = ((const uint32_t *)sl[si].ptr)[pos++];
            }
            if (i == RATE) {
                p2bb_permute(p, st);
            } else {
                if (i > 0) p2bb_permute(p, st);
                break;
            }
        }
        memcpy(digest_out, st, sizeof(uint32_t) * (size_t)OUT);
    } else {
        uint64_t st[ORC_P2_MAX_W] = {0};
        size_t si = 0, pos = 0;
        for (;;) {
            int i = 0;
            while (i < RATE) {
                while (si < nsl && pos >= sl[si].len) { ++si; pos = 0; }
                if (si >= nsl) break;
                st[i++] = ((const uint64_t *)sl[si].ptr)[pos++] % ORC_GL_P;
            }
            if (i == RATE) {
                p2gl_permute(p, st);
            } else {
                if (i > 0) p2gl_permute(p, st);
                break;
            }
        }
        memcpy(digest_out, st, sizeof(uint64_t) * (size_t)OUT);
    }
    (void)W;
}

void orc_p2_hash(const orc_p2 *p, const void *data, size_t len, void *digest_out) {
    orc_slice s = {data, len};
    orc_hash_slices(p, &s, 1, digest_out);
}

void orc_p2_compress(const orc_p2 *p, const void *left, const void *right, void *out) {
    /* truncated_permutation.hpp:61-76 */
    int D = p->digest;
    if (p->field == 0) {
        uint32_t st[ORC_P2_MAX_W] = {0};
        memcpy(st, left, sizeof(uint32_t) * (size_t)D);
        memcpy(st + D, right, sizeof(uint32_t) * (size_t)D);
        p2bb_permute(p, st);
        memcpy(out, st, sizeof(uint32_t) * (size_t)D);
    } else {
        uint64_t st[ORC_P2_MAX_W] = {0};
        memcpy(st, left, sizeof(uint64_t) * (size_t)D);
        memcpy(st + D, right, sizeof(uint64_t) * (size_t)D);
        p2gl_permute(p, st);
        memcpy(out, st, sizeof(uint64_t) * (size_t)D);
    }
}

/* ======================================================================
 * Mixed-height Merkle tree (merkle_tree.hpp:84-185)
 * ====================================================================== */
typedef struct {
    const orc_p2 *p;
    const void *const *mats;
    const size_t *widths;
    const size_t *group; /* matrix indices in hash order */
    size_t ngroup;
    size_t esize;
    unsigned char *dst; /* digests, one per row */
    const unsigned char *prev; /* optional: node digests to compress with (inject) */
} orc_rowhash_ctx;

static void orc_rowhash_range(void *vctx, size_t lo, size_t hi) {
    orc_rowhash_ctx *x = (orc_rowhash_ctx *)vctx;
    size_t dbytes = x->esize * (size_t)x->p->digest;
    orc_slice sl[256];
    for (size_t r = lo; r < hi; ++r) {
        for (size_t g = 0; g < x->ngroup; ++g) {
            size_t m = x->group[g];
            sl[g].ptr = (const unsigned char *)x->mats[m] + r * x->widths[m] * x->esize;
            sl[g].len = x->widths[m];
        }
        unsigned char rowd[ORC_P2_MAX_W * 8];
        orc_hash_slices(x->p, sl, x->ngroup, rowd);
        if (x->prev) {
            orc_p2_compress(x->p, x->prev + r * dbytes, rowd, x->dst + r * dbytes);
        } else {
            memcpy(x->dst + r * dbytes, rowd, dbytes);
        }
    }
}

typedef struct {
    const orc_p2 *p;
    const unsigned char *cur;
    unsigned char *next;
    size_t cur_size;
    size_t esize;
} orc_compress_ctx;

static void orc_compress_range(void *vctx, size_t lo, size_t hi) {
    orc_compress_ctx *x = (orc_compress_ctx *)vctx;
    size_t dbytes = x->esize * (size_t)x->p->digest;
    unsigned char zero[ORC_P2_MAX_W * 8];
    memset(zero, 0, sizeof(zero));
    for (size_t j = lo; j < hi; ++j) {
        const unsigned char *l = x->cur + 2 * j * dbytes;
        const unsigned char *r = (2 * j + 1 < x->cur_size) ? x->cur + (2 * j + 1) * dbytes : zero;
        orc_p2_compress(x->p, l, r, x->next + j * dbytes);
    }
}

int orc_mmcs_commit(const orc_p2 *p, const void *const *mats, const size_t *heights,
                    const size_t *widths, size_t n, unsigned cap_height, void *layers_out,
                    size_t layers_cap, size_t *layer_sizes, size_t max_layers, int nthreads) {
    if (n == 0 || n > 256) return -1;
    size_t esize = p->field == 0 ? 4 : 8;
    size_t dbytes = esize * (size_t)p->digest;
    /* stable sort by height descending (merkle_tree.hpp:95-100) */
    size_t *order = (size_t *)malloc(sizeof(size_t) * n);
    for (size_t i = 0; i < n; ++i) order[i] = i;
    for (size_t i = 1; i < n; ++i) { /* insertion sort is stable */
        size_t v = order[i], j = i;
        while (j > 0 && heights[order[j - 1]] < heights[v]) { order[j] = order[j - 1]; --j; }
        order[j] = v;
    }
    size_t max_h = heights[order[0]];
    if (max_h == 0 || (max_h & (max_h - 1))) { free(order); return -1; }
    size_t next_sorted = 0;
    size_t *group = (size_t *)malloc(sizeof(size_t) * n);

    unsigned char *out = (unsigned char *)layers_out;
    size_t used = 0, nl = 0;
    if (layers_cap < max_h || max_layers < 1) { free(order); free(group); return -1; }

    size_t ng = 0;
    while (next_sorted < n && heights[order[next_sorted]] == max_h) group[ng++] = order[next_sorted++];
    orc_rowhash_ctx rh = {p, mats, widths, group, ng, esize, out, NULL};
    orc_parallel(max_h, nthreads, orc_rowhash_range, &rh);
    layer_sizes[nl++] = max_h;
    used = max_h;

    size_t level = max_h, cap = (size_t)1 << cap_height;
    unsigned char *cur = out;
    while (level > cap) {
        level /= 2;
        if (used + level > layers_cap || nl >= max_layers) { free(order); free(group); return -1; }
        unsigned char *next = out + used * dbytes;
        orc_compress_ctx cc = {p, cur, next, level * 2, esize};
        orc_parallel(level, nthreads, orc_compress_range, &cc);
        ng = 0;
        while (next_sorted < n && heights[order[next_sorted]] == level) group[ng++] = order[next_sorted++];
        if (ng) {
            orc_rowhash_ctx inj = {p, mats, widths, group, ng, esize, next, next};
            orc_parallel(level, nthreads, orc_rowhash_range, &inj);
        }
        layer_sizes[nl++] = level;
        used += level;
        cur = next;
    }
    free(order);
    free(group);
    return (int)nl;
}

int orc_commit_matrix(const orc_p2 *p, const void *flat, size_t height, size_t width,
                      void *layers_out, size_t layers_cap, size_t *layer_sizes,
                      size_t max_layers, int nthreads) {
    if (width == 0 || height == 0) return -1;
    size_t esize = p->field == 0 ? 4 : 8;
    size_t dbytes = esize * (size_t)p->digest;
    unsigned char *out = (unsigned char *)layers_out;
    if (layers_cap < height || max_layers < 1) return -1;
    size_t grp = 0;
    const void *mats[1] = {flat};
    size_t widths[1] = {width};
    orc_rowhash_ctx rh = {p, mats, widths, &grp, 1, esize, out, NULL};
    orc_parallel(height, nthreads, orc_rowhash_range, &rh);
    size_t used = height, nl = 0, size = height;
    layer_sizes[nl++] = height;
    unsigned char *cur = out;
    while (size > 1) {
        size_t next_size = (size + 1) / 2;
        if (used + next_size > layers_cap || nl >= max_layers) return -1;
        unsigned char *next = out + used * dbytes;
        orc_compress_ctx cc = {p, cur, next, size, esize};
        orc_parallel(next_size, nthreads, orc_compress_range, &cc);
        layer_sizes[nl++] = next_size;
        used += next_size;
        cur = next;
        size = next_size;
    }
    return (int)nl;
}

/* ======================================================================
 * FRI fold_row / fold_matrix over BabyBear^4 (fri_folding.hpp:74-222)
 * ====================================================================== */
static void orc_fold_row(size_t index, unsigned log_height, unsigned log_arity,
                         const uint32_t beta[4], const uint32_t *evals, uint32_t out[4]) {
    if (log_arity == 0) { memcpy(out, evals, 16); return; }
    size_t arity = (size_t)1 << log_arity;
    unsigned log_folded = log_height - log_arity;
    size_t x_pow_idx = orc_rev_bits(index, log_folded);
    uint32_t omega = orc_bb_two_adic_generator(log_height);
    uint32_t x_val = orc_bb_pow(omega, x_pow_idx);
    uint32_t x[4];
    bb4_embed(x_val, x);
    uint32_t w_val = orc_bb_two_adic_generator(log_arity);
    uint32_t t[8][4];
    uint32_t w_pow = 1;
    for (size_t i = 0; i < arity; ++i) {
        uint32_t e[4];
        bb4_embed(w_pow, e);
        orc_bb4_mul(x, e, t[i]);
        w_pow = orc_bb_mul(w_pow, w_val);
    }
    for (size_t i = 0; i < arity; ++i) {
        size_t j = orc_rev_bits(i, log_arity);
        if (i < j) {
            uint32_t tmp[4];
            memcpy(tmp, t[i], 16); memcpy(t[i], t[j], 16); memcpy(t[j], tmp, 16);
        }
    }
    for (size_t i = 0; i < arity; ++i)
        if (bb4_eq(beta, t[i])) { memcpy(out, evals + 4 * i, 16); return; }
    uint32_t full_num[4] = {1, 0, 0, 0};
    for (size_t j = 0; j < arity; ++j) {
        uint32_t d[4];
        bb4_sub(beta, t[j], d);
        orc_bb4_mul(full_num, d, full_num);
    }
    uint32_t arity_inv_val = 1, two_inv = orc_bb_inv(2);
    for (unsigned k = 0; k < log_arity; ++k) arity_inv_val = orc_bb_mul(arity_inv_val, two_inv);
    uint32_t arity_inv[4];
    bb4_embed(arity_inv_val, arity_inv);
    uint32_t x_pow_am1 = orc_bb_pow(x_val, arity - 1);
    uint32_t w_inv = orc_bb_pow(w_val, arity - 1);
    uint32_t result[4] = {0, 0, 0, 0};
    uint32_t w_inv_i = 1;
    for (size_t i = 0; i < arity; ++i) {
        uint32_t bd[4], d[4], denom[4], dinv[4], L[4], tmp[4], term[4];
        bb4_embed(orc_bb_mul(x_pow_am1, w_inv_i), bd);
        bb4_sub(beta, t[i], d);
        orc_bb4_mul(d, bd, denom);
        orc_bb4_mul(full_num, arity_inv, tmp);
        orc_bb4_inv(denom, dinv);
        orc_bb4_mul(tmp, dinv, L);
        orc_bb4_mul(evals + 4 * i, L, term);
        for (int k = 0; k < 4; ++k) result[k] = orc_bb_add(result[k], term[k]);
        w_inv_i = orc_bb_mul(w_inv_i, w_inv);
    }
    memcpy(out, result, 16);
}

typedef struct {
    const uint32_t *in; uint32_t *out; unsigned log_height, log_arity; const uint32_t *beta;
} orc_fold_ctx;

static void orc_fold_range(void *vctx, size_t lo, size_t hi) {
    orc_fold_ctx *x = (orc_fold_ctx *)vctx;
    size_t arity = (size_t)1 << x->log_arity;
    for (size_t i = lo; i < hi; ++i)
        orc_fold_row(i, x->log_height, x->log_arity, x->beta, x->in + 4 * i * arity, x->out + 4 * i);
}

int orc_fold_matrix_bb4(const uint32_t *in, unsigned log_height, unsigned log_arity,
                        const uint32_t beta[4], uint32_t *out, int nthreads) {
    if (log_arity > 3 || log_arity > log_height || log_height > 27) return -1;
    size_t n = ((size_t)1 << log_height) >> log_arity;
    orc_fold_ctx x = {in, out, log_height, log_arity, beta};
    orc_parallel(n, nthreads, orc_fold_range, &x);
    return 0;
}

/* ======================================================================== */
/* PCS open: opened values and the reduced-opening vector (test oracle)     */
/* ======================================================================== */
static void bb4_add(const uint32_t a[4], const uint32_t b[4], uint32_t out[4]) {
    for (int i = 0; i < 4; ++i) out[i] = orc_bb_add(a[i], b[i]);
}
static void bb4_scale(const uint32_t a[4], uint32_t s, uint32_t out[4]) {
    for (int i = 0; i < 4; ++i) out[i] = orc_bb_mul(a[i], s);
}
static void bb4_pow(const uint32_t a[4], uint64_t e, uint32_t out[4]) {
    uint32_t r[4] = {1, 0, 0, 0}, b[4] = {a[0], a[1], a[2], a[3]};
    while (e) {
        if (e & 1) orc_bb4_mul(r, b, r);
        orc_bb4_mul(b, b, b);
        e >>= 1;
    }
    memcpy(out, r, sizeof r);
}

typedef struct {
    const uint32_t *lde;
    unsigned log_n;
    size_t w;
    uint32_t shift;
    const uint32_t *z;
    uint32_t *partial; /* per row block: w x 4 partial sums */
    size_t block;
} orc_open_ctx;

/* rows [b*block, (b+1)*block) of sum_i d_i f_i / (z - g h_i) */
static void orc_open_range(void *vx, size_t b0, size_t b1) {
    orc_open_ctx *x = (orc_open_ctx *)vx;
    const size_t n = (size_t)1 << x->log_n;
    const uint32_t om = orc_bb_two_adic_generator(x->log_n);
    /* common_inv = 1 / (n g^(n-1)) (interpolation.hpp compute_diff_invs) */
    const uint32_t common_inv = orc_bb_inv(orc_bb_mul((uint32_t)(n % ORC_BB_P), orc_bb_pow(x->shift, n - 1)));
    for (size_t b = b0; b < b1; ++b) {
        uint32_t *acc = x->partial + b * x->w * 4;
        memset(acc, 0, x->w * 4 * sizeof(uint32_t));
        const size_t r0 = b * x->block, r1 = r0 + x->block < n ? r0 + x->block : n;
        uint32_t h = orc_bb_pow(om, r0);
        for (size_t i = r0; i < r1; ++i) {
            const uint32_t d = orc_bb_mul(h, common_inv);
            uint32_t diff[4] = {orc_bb_sub(x->z[0], orc_bb_mul(x->shift, h)), x->z[1], x->z[2], x->z[3]}, inv[4];
            orc_bb4_inv(diff, inv);
            for (size_t c = 0; c < x->w; ++c) {
                uint32_t t[4];
                bb4_scale(inv, orc_bb_mul(x->lde[i * x->w + c], d), t);
                bb4_add(acc + 4 * c, t, acc + 4 * c);
            }
            h = orc_bb_mul(h, om);
        }
    }
}

void orc_pcs_open_values(const uint32_t *lde, unsigned log_n, size_t w, uint32_t shift,
                         const uint32_t z[4], uint32_t *out, int nthreads) {
    const size_t n = (size_t)1 << log_n, block = 256;
    const size_t nb = (n + block - 1) / block;
    uint32_t *partial = (uint32_t *)malloc(nb * w * 4 * sizeof(uint32_t));
    orc_open_ctx x = {lde, log_n, w, shift, z, partial, block};
    orc_parallel(nb, nthreads, orc_open_range, &x);
    /* vanishing factor z^n - g^n */
    uint32_t van[4];
    bb4_pow(z, n, van);
    van[0] = orc_bb_sub(van[0], orc_bb_pow(shift, n));
    for (size_t c = 0; c < w; ++c) {
        uint32_t s[4] = {0, 0, 0, 0};
        for (size_t b = 0; b < nb; ++b) bb4_add(s, partial + (b * w + c) * 4, s);
        orc_bb4_mul(van, s, out + 4 * c);
    }
    free(partial);
}

typedef struct {
    const uint32_t *lde;
    unsigned log_n;
    size_t w;
    uint32_t shift;
    const uint32_t *z;
    size_t m;
    const uint32_t *opened;
    const uint32_t *apow; /* m*w alpha powers */
    uint32_t *q;
} orc_reduce_ctx;

static void orc_reduce_range(void *vx, size_t k0, size_t k1) {
    orc_reduce_ctx *x = (orc_reduce_ctx *)vx;
    const uint32_t om = orc_bb_two_adic_generator(x->log_n);
    uint32_t xk = orc_bb_mul(x->shift, orc_bb_pow(om, k0));
    for (size_t k = k0; k < k1; ++k) {
        for (size_t p = 0; p < x->m; ++p) {
            const uint32_t *zp = x->z + 4 * p;
            uint32_t diff[4] = {orc_bb_sub(zp[0], xk), zp[1], zp[2], zp[3]}, dinv[4];
            orc_bb4_inv(diff, dinv);
            for (size_t c = 0; c < x->w; ++c) {
                const uint32_t *fz = x->opened + 4 * (p * x->w + c);
                uint32_t numer[4] = {orc_bb_sub(fz[0], x->lde[k * x->w + c]), fz[1], fz[2], fz[3]}, t[4];
                orc_bb4_mul(x->apow + 4 * (p * x->w + c), numer, t);
                orc_bb4_mul(t, dinv, t);
                bb4_add(x->q + 4 * k, t, x->q + 4 * k);
            }
        }
        xk = orc_bb_mul(xk, om);
    }
}

void orc_pcs_reduce(const uint32_t *lde, unsigned log_n, size_t w, uint32_t shift,
                    const uint32_t *z, size_t m, const uint32_t *opened, const uint32_t alpha[4],
                    uint64_t ap0, uint32_t *q, int nthreads) {
    const size_t n = (size_t)1 << log_n;
    uint32_t *apow = (uint32_t *)malloc((m * w + 1) * 4 * sizeof(uint32_t));
    bb4_pow(alpha, ap0, apow);
    for (size_t i = 1; i < m * w; ++i) orc_bb4_mul(apow + 4 * (i - 1), alpha, apow + 4 * i);
    orc_reduce_ctx x = {lde, log_n, w, shift, z, m, opened, apow, q};
    orc_parallel(n, nthreads, orc_reduce_range, &x);
    free(apow);
}
