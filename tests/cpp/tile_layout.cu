// Host-only check of the in-CTA transform's shared-memory index arithmetic
// (plonky3-gpu_gb300/csrc/ntt.cuh), for every tile shape the kernels use:
//  * DftShape::at(row0(base, c), mk) == addr(base + mk, c) for the rows each
//    super-stage, the last super-stage's tile store and the first
//    super-stage's bit-reversed read touch (base and mk share no set bit);
//  * the stage-ordered twiddle table: entry off_J + i_lo * R + s holds the
//    exponent (i_lo * bitrev(s)) << TWS_J of super-stage J, and the table has
//    exactly ss_tw_size entries.
// Prints the number of mismatches; exits non-zero on any.
#include <cstdio>

#include "ntt.cuh"

using namespace p3g;

template <class T, int LOGN, int C>
static int check_addr() {
    using SH = DftShape<T, LOGN, C, 256>;
    constexpr int MLR = ss_max_lr<T>();
    int bad = 0;
    for (int J = 0; J < ss_count(LOGN, MLR); ++J) {
        const int LR = ss_radix(LOGN, J, MLR), LS = LOGN - ss_consumed(LOGN, J, MLR);
        const int R = 1 << LR, M = (1 << LS) >> LR, GROUPS = (1 << LOGN) >> LR;
        for (int g = 0; g < GROUPS; ++g)
            for (int c = 0; c < C; ++c) {
                const int base = (g / M) * (1 << LS) + g % M;
                for (int k = 0; k < R; ++k) {
                    bad += SH::at(SH::row0(base, c), M * k) != SH::addr(base + M * k, c);
                    if (J == 0) {
                        const int b = int(bitrev_ct(unsigned(base), LOGN));
                        bad += SH::at(SH::row0(b, c), int(bitrev_ct(unsigned(M * k), LOGN))) !=
                               SH::addr(int(bitrev_ct(unsigned(base + M * k), LOGN)), c);
                    }
                }
            }
    }
    return bad;
}

static int check_tw(int logn, int mlr) {
    int bad = 0, seen = 0;
    for (int J = 0; J + 1 < ss_count(logn, mlr); ++J) {
        const int LR = ss_radix(logn, J, mlr), LS = logn - ss_consumed(logn, J, mlr);
        const int R = 1 << LR, M = (1 << LS) >> LR;
        for (int i_lo = 0; i_lo < M; ++i_lo)
            for (int s = 0; s < R; ++s, ++seen) {
                const int idx = ss_tw_off(logn, J, mlr) + i_lo * R + s;
                const uint32_t e = uint32_t((i_lo * int(bitrev_ct(unsigned(s), LR))) << (logn - LS));
                bad += idx >= ss_tw_size(logn, mlr) || ss_tw_exp(logn, mlr, idx) != e;
            }
    }
    return bad + (seen != ss_tw_size(logn, mlr));
}

#define SHAPES(T, L) check_addr<T, L, 4>() + check_addr<T, L, 8>() + check_addr<T, L, 16>() + check_addr<T, L, 32>()
int main() {
    int bad = SHAPES(uint32_t, 1) + SHAPES(uint32_t, 2) + SHAPES(uint32_t, 3) + SHAPES(uint32_t, 4) +
              SHAPES(uint32_t, 5) + SHAPES(uint32_t, 6) + SHAPES(uint32_t, 7) + SHAPES(uint32_t, 8) +
              SHAPES(uint32_t, 9) + SHAPES(uint32_t, 10) + SHAPES(uint32_t, 11);
    bad += SHAPES(uint64_t, 1) + SHAPES(uint64_t, 2) + SHAPES(uint64_t, 3) + SHAPES(uint64_t, 4) +
           SHAPES(uint64_t, 5) + SHAPES(uint64_t, 6) + SHAPES(uint64_t, 7) + SHAPES(uint64_t, 8) +
           SHAPES(uint64_t, 9) + SHAPES(uint64_t, 10) + SHAPES(uint64_t, 11);
    for (int L = 1; L <= 11; ++L) bad += check_tw(L, ss_max_lr<uint32_t>()) + check_tw(L, ss_max_lr<uint64_t>());
    printf("mismatches %d\n", bad);
    return bad != 0;
}
