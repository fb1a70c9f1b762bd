// lde_bb.cu -- BabyBear instantiation of the coset LDE (lde.cuh).
#include "lde.cuh"

namespace p3g {

void lde_bb(p3g_ctx* ctx, const uint32_t* in, int log_h, int w, int log_b, uint32_t shift, int bitrev_out,
            uint32_t* out, cudaStream_t st) {
    lde_impl<FBB>(ctx, in, log_h, w, log_b, shift, bitrev_out, out, st, ctx->bb_roots());
}
}  // namespace p3g
