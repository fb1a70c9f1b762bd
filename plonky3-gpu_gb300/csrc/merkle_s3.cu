// merkle_s3.cu -- instantiates the Merkle kernels for one Poseidon2 schedule
// (BabyBear width 16, x^5, 8 full + 14 partial rounds).
#define P3G_MERKLE_INSTANTIATE
#include "merkle.cuh"

namespace p3g {
template struct Launch<HBB, 5, 8, 14>;
}  // namespace p3g
