// lde_gl.cu -- Goldilocks instantiation of the coset LDE (lde.cuh).
#include "lde.cuh"

namespace p3g {

void lde_gl(p3g_ctx* ctx, const uint64_t* in, int log_h, int w, int log_b, uint64_t shift, int bitrev_out,
            uint64_t* out, cudaStream_t st) {
    lde_impl<FGL>(ctx, in, log_h, w, log_b, shift, bitrev_out, out, st, ctx->gl_roots(),
                  static_cast<const FGL::TW*>(ctx->gl_dft_tw));
}

void* make_dft_tw_gl() {
    const auto v = build_dft_tw<FGL>();
    void* d = nullptr;
    P3G_CUDA(cudaMalloc(&d, v.size() * sizeof(v[0])));
    P3G_CUDA(cudaMemcpy(d, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice));
    return d;
}

}  // namespace p3g
