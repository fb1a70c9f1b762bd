// lde_noalloc.cu -- a BabyBear coset LDE entry point that allocates nothing.
//
// Who needs it: callers that must not enter the CUDA allocator during a
// proof.  A prover service that reserves its HBM budget at start-up (so that
// a request can never fail, stall or fragment the heap on an allocation in
// the middle of a commitment), or a host that embeds the library inside its
// own device-memory manager, cannot accept the stream-ordered pool
// allocations that p3g_coset_lde makes for its scratch.  This variant runs
// the same kernels (lde.cuh) with every scratch buffer carved out of one
// file-scope device array, and reads the root-of-unity tables from two more
// file-scope device arrays, so it needs neither a context nor any
// allocation.
//
// Costs and rules:
//  * every GPU that loads the library holds these arrays (16 MiB of scratch
//    plus 96 KiB of root tables) until the process exits;
//  * the first call on a device does a one-time set-up with that device
//    current: it resolves the arrays' device addresses with
//    cudaGetSymbolAddress (host code must never pass the array names
//    themselves to a kernel -- in host code they are host-side stand-ins,
//    not device addresses) and fills the root tables with a synchronous
//    copy.  Make that first call before any stream capture;
//  * all calls share the one scratch array, which keeps the last call's
//    contents: calls that may overlap on the GPU (different streams, or
//    different host threads) race and must be serialised by the caller.
//    Nothing in the scratch needs to start at zero: every word a call reads
//    was written earlier in the same call;
//  * sizes beyond the scratch maximum are rejected with P3G_EINVAL.
#include <mutex>

#include "lde.cuh"

namespace p3g {
namespace {

constexpr size_t NOALLOC_SCRATCH_WORDS = size_t(4) << 20;  // 16 MiB of BabyBear words
constexpr int NA_LB = RootTab<FBB>::LB;

static __device__ __align__(256) uint32_t g_na_scratch[NOALLOC_SCRATCH_WORDS];
static __device__ __align__(256) uint32_t g_na_roots_lo[1u << NA_LB];
static __device__ __align__(256) uint32_t g_na_roots_hi[1u << (27 - NA_LB)];

struct NoAllocDevice {
    bool ready = false;
    uint32_t* scratch = nullptr;
    uint32_t* lo = nullptr;
    uint32_t* hi = nullptr;
};
std::mutex g_na_mu;
NoAllocDevice g_na_dev[128];

// One-time set-up for the current device: device addresses of the arrays and
// the contents of the root tables.
const NoAllocDevice& na_setup() {
    int dev = 0;
    P3G_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) throw Error(P3G_EUNSUPPORTED, "coset_lde_bb_noalloc: device index out of range");
    std::lock_guard<std::mutex> lk(g_na_mu);
    NoAllocDevice& d = g_na_dev[dev];
    if (d.ready) return d;
    P3G_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&d.scratch), g_na_scratch));
    P3G_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&d.lo), g_na_roots_lo));
    P3G_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&d.hi), g_na_roots_hi));
    std::vector<uint32_t> lo(size_t(1) << NA_LB), hi(size_t(1) << (27 - NA_LB));
    const uint32_t g27 = bb::two_adic_generator(27);
    uint32_t v = 1;
    for (auto& x : lo) {
        x = bb::to_mont(v);
        v = bb::h_mul(v, g27);
    }
    const uint32_t step = v;
    v = 1;
    for (auto& x : hi) {
        x = bb::to_mont(v);
        v = bb::h_mul(v, step);
    }
    P3G_CUDA(cudaMemcpy(d.lo, lo.data(), lo.size() * 4, cudaMemcpyHostToDevice));
    P3G_CUDA(cudaMemcpy(d.hi, hi.data(), hi.size() * 4, cudaMemcpyHostToDevice));
    d.ready = true;
    return d;
}

void lde_bb_noalloc(const uint32_t* in, int log_h, int w, int log_b, uint32_t shift, int bitrev_out,
                    uint32_t* out, cudaStream_t st) {
    using F = FBB;
    P3G_REQUIRE(log_h >= 0 && log_b >= 0, "coset_lde_bb_noalloc: negative size");
    P3G_REQUIRE(log_h + log_b <= 27, "coset_lde_bb_noalloc: log_h + log_blowup exceeds two-adicity");
    P3G_REQUIRE(shift % bb::P != 0 && shift < bb::P, "coset_lde_bb_noalloc: shift must be canonical and non-zero");
    if (log_h > LDE_PASS_MAX) throw Error(P3G_EUNSUPPORTED, "coset_lde_bb_noalloc: log_h > 21 is not supported");
    if (w == 0) return;
    // scratch this call needs (power tables, prepared twists, pass-1 output,
    // natural-order staging), carved from the fixed array in 256-byte steps
    const LdeScratch need = lde_scratch<F>(log_h, w, log_b, bitrev_out);
    if (need.total() > NOALLOC_SCRATCH_WORDS * 4)
        throw Error(P3G_EINVAL, "coset_lde_bb_noalloc: needs " + std::to_string(need.total()) +
                                    " bytes of scratch, more than its fixed maximum of " +
                                    std::to_string(NOALLOC_SCRATCH_WORDS * 4) + " bytes");
    const NoAllocDevice& d = na_setup();
    void* buf[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    unsigned char* next = reinterpret_cast<unsigned char*>(d.scratch);
    for (int i = 0; i < 5; ++i) {
        if (!need.bytes[i]) continue;
        buf[i] = next;
        next += LdeScratch::round(need.bytes[i]);
    }
    // no prepared twiddle table: the kernels derive their twiddles from the roots
    lde_run<F>(in, log_h, w, log_b, shift, bitrev_out, out, st, RootTab<F>{d.lo, d.hi}, nullptr, buf);
}

}  // namespace
}  // namespace p3g

extern "C" int p3g_coset_lde_bb_noalloc(const void* d_in, uint32_t log_h, uint32_t width, uint32_t log_blowup,
                                        uint32_t shift, int bitrev_out, void* d_out, void* stream) {
    try {
        P3G_REQUIRE(width == 0 || (d_in && d_out), "coset_lde_bb_noalloc: null argument");
        P3G_REQUIRE(width <= (1u << 24), "coset_lde_bb_noalloc: width too large");
        p3g::lde_bb_noalloc(static_cast<const uint32_t*>(d_in), int(log_h), int(width), int(log_blowup), shift,
                            bitrev_out, static_cast<uint32_t*>(d_out), static_cast<cudaStream_t>(stream));
    } catch (const p3g::Error& e) {
        p3g::set_last_error(e.what());
        return e.status;
    } catch (const std::exception& e) {
        p3g::set_last_error(e.what());
        return P3G_ECUDA;
    }
    return P3G_OK;
}
