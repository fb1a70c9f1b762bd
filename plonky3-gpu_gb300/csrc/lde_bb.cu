// lde_bb.cu -- BabyBear instantiation of the coset LDE (lde.cuh).
#include "lde.cuh"

namespace p3g {

void lde_bb(p3g_ctx* ctx, const uint32_t* in, int log_h, int w, int log_b, uint32_t shift, int bitrev_out,
            uint32_t* out, cudaStream_t st) {
    lde_impl<FBB>(ctx, in, log_h, w, log_b, shift, bitrev_out, out, st, ctx->bb_roots(),
                  static_cast<const FBB::TW*>(ctx->bb_dft_tw));
}

void* make_dft_tw_bb() {
    const auto v = build_dft_tw<FBB>();
    void* d = nullptr;
    P3G_CUDA(cudaMalloc(&d, v.size() * sizeof(v[0])));
    P3G_CUDA(cudaMemcpy(d, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice));
    return d;
}

}  // namespace p3g
