// merkle_s1.cu -- instantiates the Merkle kernels for one Poseidon2 schedule
// (BabyBear width 16, x^7, 8 full + 13 partial rounds).
#define P3G_MERKLE_INSTANTIATE
#include "merkle.cuh"

namespace p3g {
template struct Launch<HBB, 7, 8, 13>;
}  // namespace p3g
