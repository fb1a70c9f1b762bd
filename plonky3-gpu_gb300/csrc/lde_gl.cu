// lde_gl.cu -- Goldilocks instantiation of the coset LDE (lde.cuh).
#include "lde.cuh"

namespace p3g {

void lde_gl(p3g_ctx* ctx, const uint64_t* in, int log_h, int w, int log_b, uint64_t shift, int bitrev_out,
            uint64_t* out, cudaStream_t st) {
    lde_impl<FGL>(ctx, in, log_h, w, log_b, shift, bitrev_out, out, st, ctx->gl_roots(),
                  static_cast<const FGL::TW*>(ctx->gl_dft_tw));
}

size_t lde_group_table_bytes_gl(int log_h, int log_b, int k) { return lde_table_bytes<FGL>(log_h, log_b)[k]; }
size_t lde_group_scr_bytes_gl(int log_h, int w) { return sizeof(uint64_t) * lde_scr_elems<FGL>(log_h, w); }
void lde_group_tables_gl(p3g_ctx* ctx, int log_h, int log_b, uint64_t shift, void* const* tab, cudaStream_t st) {
    lde_tables<FGL>(log_h, log_b, shift % FGL::P, tab, ctx->gl_roots(), st);
}
void lde_group_gl(p3g_ctx* ctx, int log_h, int log_b, const void* const* in, void* const* scr, void* const* out,
                  const uint32_t* w, size_t n, void* const* tab, cudaStream_t st) {
    lde_group_t<FGL>(log_h, log_b, in, scr, out, w, n, tab, ctx->gl_roots(),
                    static_cast<const FGL::TW*>(ctx->gl_dft_tw), st);
}

void* make_dft_tw_gl() {
    const auto v = build_dft_tw<FGL>();
    void* d = nullptr;
    P3G_CUDA(cudaMalloc(&d, v.size() * sizeof(v[0])));
    P3G_CUDA(cudaMemcpy(d, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice));
    return d;
}

}  // namespace p3g
