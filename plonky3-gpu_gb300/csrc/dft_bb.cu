// dft_bb.cu -- BabyBear instantiation of the dft / idft / coset variants (dft.cuh).
#include "dft.cuh"

namespace p3g {

void dft_bb(p3g_ctx* ctx, int kind, const uint32_t* in, int log_h, int w, uint32_t shift, int bitrev_out,
            uint32_t* out, cudaStream_t st) {
    dft_impl<FBB>(ctx, kind, in, log_h, w, shift, bitrev_out, out, st, ctx->bb_roots(),
                  static_cast<const FBB::TW*>(ctx->bb_dft_tw));
}

void lde_big(p3g_ctx* ctx, const uint32_t* in, int log_h, int w, int log_b, uint64_t shift, int bitrev_out,
             uint32_t* out, cudaStream_t st) {
    lde_big_run<FBB>(ctx, in, log_h, w, log_b, shift, bitrev_out, out, st, ctx->bb_roots(),
                     static_cast<const FBB::TW*>(ctx->bb_dft_tw));
}

}  // namespace p3g
