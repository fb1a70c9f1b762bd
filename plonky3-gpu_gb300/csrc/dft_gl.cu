// dft_gl.cu -- Goldilocks instantiation of the dft / idft / coset variants (dft.cuh).
#include "dft.cuh"

namespace p3g {

void dft_gl(p3g_ctx* ctx, int kind, const uint64_t* in, int log_h, int w, uint64_t shift, int bitrev_out,
            uint64_t* out, cudaStream_t st) {
    dft_impl<FGL>(ctx, kind, in, log_h, w, shift, bitrev_out, out, st, ctx->gl_roots(),
                  static_cast<const FGL::TW*>(ctx->gl_dft_tw));
}

void lde_big(p3g_ctx* ctx, const uint64_t* in, int log_h, int w, int log_b, uint64_t shift, int bitrev_out,
             uint64_t* out, cudaStream_t st) {
    lde_big_run<FGL>(ctx, in, log_h, w, log_b, shift, bitrev_out, out, st, ctx->gl_roots(),
                     static_cast<const FGL::TW*>(ctx->gl_dft_tw));
}

}  // namespace p3g
