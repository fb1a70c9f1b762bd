// merkle_s2.cu -- instantiates the Merkle kernels for one Poseidon2 schedule
// (BabyBear width 16, x^7, 8 full + 22 partial rounds).
#define P3G_MERKLE_INSTANTIATE
#include "merkle.cuh"

namespace p3g {
template struct Launch<HBB, 7, 8, 22>;
}  // namespace p3g
