// plan.cu -- the batched commit as one CUDA graph.
//
// A plan fixes a batch of traces (device pointers and shapes), allocates
// every output once (the bit-reversed LDE of each trace, the digest layers,
// the injected-row digests, the row-hash work descriptors), and captures the
// whole commitment -- every LDE spread over several streams, the persistent
// row-hash kernel over all height groups, each tree level, and optionally a
// FRI fold -- into one graph.  p3g_plan_launch replays it with a single
// cudaGraphLaunch; refill the trace buffers between launches to commit new
// data of the same shapes.  This is the batched form of
// TwoAdicFriPcs::commit's LDE + MerkleTreeMmcs::commit (two_adic_fri_pcs.hpp:207-266,
// merkle_tree_mmcs.hpp:100-107) followed by fold_matrix (fri_folding.hpp:200).
//
// Stream count: the LDEs are list-scheduled (largest first onto the least
// loaded stream) over k streams.  With k = 0 an autotuner captures k in
// {1, 2, 4, 8}, times two launches of each and keeps the fastest; decisions
// are cached per (field, number of traces, log2 of LDE elements) in memory
// and, when P3G_TUNE_CACHE names a file, in that JSON file.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>

#include "internal.hpp"

struct p3g_plan {
    int field = 0;
    p3g_tree tree;
    std::vector<p3g_trace> traces;
    bool has_fold = false;
    p3g_fold_job fold{};
    uint32_t cap_height = 0;
    int nstreams = 1;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t kernels_per_launch = 0;
};

namespace p3g {
namespace {

struct Streams {
    std::vector<cudaStream_t> s;
    std::vector<cudaEvent_t> e;
    explicit Streams(int n) {
        s.resize(n);
        e.resize(n + 1);
        for (auto& x : s) P3G_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
        for (auto& x : e) P3G_CUDA(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
    }
    ~Streams() {
        for (auto x : s) cudaStreamDestroy(x);
        for (auto x : e) cudaEventDestroy(x);
    }
};

// Captures the plan's device work with `k` LDE streams into plan->graph/exec.
void capture(p3g_ctx* ctx, p3g_plan* plan, int k) {
    Streams ss(k + 1);  // s[0] is the capture origin and runs the tree build
    cudaStream_t s0 = ss.s[0];
    const uint64_t l0 = 0;
    (void)l0;
    P3G_CUDA(cudaStreamBeginCapture(s0, cudaStreamCaptureModeRelaxed));
    try {
        P3G_CUDA(cudaEventRecord(ss.e[0], s0));
        for (int i = 1; i <= k; ++i) P3G_CUDA(cudaStreamWaitEvent(ss.s[i], ss.e[0], 0));
        // list scheduling: largest LDE first onto the least loaded stream
        std::vector<size_t> order(plan->traces.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = i;
        auto work = [&](size_t i) {
            const auto& t = plan->traces[i];
            return (uint64_t(1) << (t.log_h + t.log_blowup)) * t.width;
        };
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return work(a) > work(b); });
        std::vector<uint64_t> load(k, 0);
        for (size_t i : order) {
            const int j = int(std::min_element(load.begin(), load.end()) - load.begin());
            load[j] += work(i) + 1;
            const auto& t = plan->traces[i];
            cudaStream_t st = ss.s[1 + j];
            if (plan->field == P3G_BABYBEAR)
                lde_bb(ctx, static_cast<const uint32_t*>(t.d_trace), int(t.log_h), int(t.width), int(t.log_blowup),
                       uint32_t(t.shift), 1, static_cast<uint32_t*>(plan->tree.owned[i]), st);
            else
                lde_gl(ctx, static_cast<const uint64_t*>(t.d_trace), int(t.log_h), int(t.width), int(t.log_blowup),
                       t.shift, 1, static_cast<uint64_t*>(plan->tree.owned[i]), st);
        }
        if (plan->has_fold) {
            const auto& f = plan->fold;
            fold_bb4(ctx, static_cast<const uint32_t*>(f.d_in), int(f.log_height), int(f.log_arity), f.beta,
                     static_cast<uint32_t*>(f.d_out), ss.s[1 + (k > 1 ? k - 1 : 0)]);
        }
        for (int i = 1; i <= k; ++i) {
            P3G_CUDA(cudaEventRecord(ss.e[i], ss.s[i]));
            P3G_CUDA(cudaStreamWaitEvent(s0, ss.e[i], 0));
        }
        tree_enqueue(ctx, &plan->tree, s0);
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(s0, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    cudaGraph_t g = nullptr;
    P3G_CUDA(cudaStreamEndCapture(s0, &g));
    cudaGraphExec_t ex = nullptr;
    cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        P3G_CUDA(e);
    }
    size_t nnodes = 0;
    P3G_CUDA(cudaGraphGetNodes(g, nullptr, &nnodes));
    std::vector<cudaGraphNode_t> nodes(nnodes);
    P3G_CUDA(cudaGraphGetNodes(g, nodes.data(), &nnodes));
    uint64_t kernels = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType ty;
        P3G_CUDA(cudaGraphNodeGetType(nd, &ty));
        if (ty == cudaGraphNodeTypeKernel) ++kernels;
    }
    if (plan->exec) cudaGraphExecDestroy(plan->exec);
    if (plan->graph) cudaGraphDestroy(plan->graph);
    plan->graph = g;
    plan->exec = ex;
    plan->kernels_per_launch = kernels;
    plan->nstreams = k;
}

float time_launches(p3g_plan* plan, int reps) {
    cudaStream_t st;
    P3G_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cudaEvent_t a, b;
    P3G_CUDA(cudaEventCreate(&a));
    P3G_CUDA(cudaEventCreate(&b));
    P3G_CUDA(cudaGraphLaunch(plan->exec, st));  // warm
    P3G_CUDA(cudaEventRecord(a, st));
    for (int i = 0; i < reps; ++i) P3G_CUDA(cudaGraphLaunch(plan->exec, st));
    P3G_CUDA(cudaEventRecord(b, st));
    P3G_CUDA(cudaEventSynchronize(b));
    float ms = 0;
    P3G_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaStreamDestroy(st);
    return ms / float(reps);
}

// --------------------------------------------------------------- tuning cache
std::mutex g_tune_mu;
std::map<std::string, int> g_tune;
bool g_tune_loaded = false;

std::string tune_path() {
    const char* p = std::getenv("P3G_TUNE_CACHE");
    return p ? std::string(p) : std::string();
}
void tune_load() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const std::string path = tune_path();
    if (path.empty()) return;
    std::ifstream in(path);
    std::string line;
    // one entry per line: "key": streams,
    while (std::getline(in, line)) {
        const size_t a = line.find('"'), b = line.find('"', a + 1), c = line.find(':', b);
        if (a == std::string::npos || b == std::string::npos || c == std::string::npos) continue;
        g_tune[line.substr(a + 1, b - a - 1)] = std::atoi(line.c_str() + c + 1);
    }
}
void tune_store() {
    const std::string path = tune_path();
    if (path.empty()) return;
    std::ofstream out(path, std::ios::trunc);
    out << "{\n";
    size_t i = 0;
    for (const auto& kv : g_tune) out << "  \"" << kv.first << "\": " << kv.second << (++i < g_tune.size() ? ",\n" : "\n");
    out << "}\n";
}
std::string tune_key(const p3g_plan* plan) {
    uint64_t elems = 0;
    for (const auto& t : plan->traces) elems += (uint64_t(1) << (t.log_h + t.log_blowup)) * t.width;
    int lg = 0;
    while ((uint64_t(1) << (lg + 1)) <= elems) ++lg;
    std::ostringstream k;
    k << "commit/f" << plan->field << "/n" << plan->traces.size() << "/e2^" << lg << (plan->has_fold ? "/fold" : "");
    return k.str();
}

}  // namespace
}  // namespace p3g

extern "C" {

int p3g_plan_commit(p3g_ctx* ctx, int field, const p3g_trace* traces, size_t n_traces, uint32_t cap_height,
                    const p3g_fold_job* fold, uint32_t n_streams, p3g_plan** out) {
    try {
        P3G_REQUIRE(ctx && traces && n_traces > 0 && out, "plan_commit: null argument");
        P3G_REQUIRE(field == P3G_BABYBEAR || field == P3G_GOLDILOCKS, "plan_commit: unknown field");
        P3G_REQUIRE(!fold || field == P3G_BABYBEAR, "plan_commit: the fold is over BabyBear^4");
        P3G_REQUIRE(n_streams <= 16, "plan_commit: at most 16 streams");
        int prev = 0;
        cudaGetDevice(&prev);
        if (prev != ctx->device) P3G_CUDA(cudaSetDevice(ctx->device));
        auto plan = std::make_unique<p3g_plan>();
        plan->field = field;
        plan->cap_height = cap_height;
        plan->traces.assign(traces, traces + n_traces);
        plan->tree.field = field;
        plan->tree.in_plan = true;
        if (fold) {
            plan->has_fold = true;
            plan->fold = *fold;
        }
        const size_t esz = field == P3G_BABYBEAR ? 4 : 8;
        cudaStream_t st0 = nullptr;
        try {
            for (const auto& t : plan->traces) {
                P3G_REQUIRE(t.width == 0 || t.d_trace, "plan_commit: null trace");
                P3G_REQUIRE(t.log_h + t.log_blowup <= (field == P3G_BABYBEAR ? 27u : 32u),
                            "plan_commit: log_h + log_blowup exceeds two-adicity");
                const uint64_t H = uint64_t(1) << (t.log_h + t.log_blowup);
                void* lde = ctx->alloc(esz * H * std::max<uint32_t>(t.width, 1), st0);
                plan->tree.owned.push_back(lde);
                plan->tree.mats.push_back(p3g_matrix{lde, H, t.width, 0});
            }
            p3g::tree_prepare(ctx, &plan->tree, cap_height, false, st0, true);
            if (n_streams > 0) {
                p3g::capture(ctx, plan.get(), int(n_streams));
            } else {
                std::lock_guard<std::mutex> lk(p3g::g_tune_mu);
                p3g::tune_load();
                const std::string key = p3g::tune_key(plan.get());
                auto it = p3g::g_tune.find(key);
                if (it != p3g::g_tune.end()) {
                    p3g::capture(ctx, plan.get(), it->second);
                } else {
                    int best = 1;
                    float best_ms = 1e30f;
                    for (int k : {1, 2, 4, 8}) {
                        if (k > int(n_traces) && k > 1) break;
                        p3g::capture(ctx, plan.get(), k);
                        const float ms = p3g::time_launches(plan.get(), 2);
                        if (ms < best_ms) {
                            best_ms = ms;
                            best = k;
                        }
                    }
                    p3g::g_tune[key] = best;
                    p3g::tune_store();
                    p3g::capture(ctx, plan.get(), best);
                }
            }
            P3G_CUDA(cudaDeviceSynchronize());
        } catch (...) {
            if (plan->exec) cudaGraphExecDestroy(plan->exec);
            if (plan->graph) cudaGraphDestroy(plan->graph);
            p3g::tree_release(ctx, &plan->tree, st0);
            throw;
        }
        *out = plan.release();
        if (prev != ctx->device) cudaSetDevice(prev);
    } catch (const p3g::Error& e) {
        p3g::set_last_error(e.what());
        return e.status;
    } catch (const std::exception& e) {
        p3g::set_last_error(e.what());
        return P3G_ECUDA;
    }
    return P3G_OK;
}

int p3g_plan_launch(p3g_ctx* ctx, p3g_plan* plan, void* stream) {
    try {
        P3G_REQUIRE(ctx && plan && plan->exec, "plan_launch: null argument");
        P3G_CUDA(cudaGraphLaunch(plan->exec, static_cast<cudaStream_t>(stream)));
        for (uint64_t i = 0; i < plan->kernels_per_launch; ++i) p3g::count_launch();
    } catch (const p3g::Error& e) {
        p3g::set_last_error(e.what());
        return e.status;
    }
    return P3G_OK;
}

int p3g_plan_info(const p3g_plan* plan, const p3g_tree** tree, uint32_t* n_streams, uint64_t* kernels_per_launch) {
    if (!plan) {
        p3g::set_last_error("plan_info: null plan");
        return P3G_EINVAL;
    }
    if (tree) *tree = &plan->tree;
    if (n_streams) *n_streams = uint32_t(plan->nstreams);
    if (kernels_per_launch) *kernels_per_launch = plan->kernels_per_launch;
    return P3G_OK;
}

int p3g_plan_destroy(p3g_ctx* ctx, p3g_plan* plan) {
    try {
        if (!plan) return P3G_OK;
        P3G_REQUIRE(ctx, "plan_destroy: null context");
        P3G_CUDA(cudaDeviceSynchronize());
        if (plan->exec) cudaGraphExecDestroy(plan->exec);
        if (plan->graph) cudaGraphDestroy(plan->graph);
        p3g::tree_release(ctx, &plan->tree, nullptr);
        P3G_CUDA(cudaDeviceSynchronize());
        delete plan;
    } catch (const p3g::Error& e) {
        p3g::set_last_error(e.what());
        return e.status;
    }
    return P3G_OK;
}

}  // extern "C"
