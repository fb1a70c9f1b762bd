// merkle_s4.cu -- instantiates the Merkle kernels for one Poseidon2 schedule
// (Goldilocks width 8, x^7, 8 full + 22 partial rounds).
#define P3G_MERKLE_INSTANTIATE
#include "merkle.cuh"

namespace p3g {
template struct Launch<HGL, 7, 8, 22>;
}  // namespace p3g
