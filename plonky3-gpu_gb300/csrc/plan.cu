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
// A host-input plan (p3g_plan_commit_host) takes the traces and the fold
// input in pinned host memory: the graph copies each one into a device buffer
// the plan owns, on a copy stream, in the order the LDE streams consume them,
// and each LDE waits only for its own trace's copy, so the copies overlap the
// LDEs of the traces copied before.
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
#include <tuple>

#include "internal.hpp"

struct p3g_plan {
    int field = 0;
    p3g_tree tree;
    std::vector<p3g_trace> traces;
    bool has_fold = false;
    p3g_fold_job fold{};
    // host-input plans: device copies of the traces and of the fold input
    bool host_input = false;
    std::vector<void*> d_traces;
    void* d_fold_in = nullptr;
    // the LDE shape groups, their tables and scratch prepared once
    std::vector<p3g::LdeGroup> groups;
    bool grouped = true;
    uint32_t cap_height = 0;
    int nstreams = 1;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t kernels_per_launch = 0;
};

namespace p3g {

// ------------------------------------------------------------ LDE groups
std::vector<LdeGroup> lde_groups(const p3g_trace* traces, size_t n) {
    std::vector<LdeGroup> out;
    std::map<std::tuple<uint32_t, uint32_t, uint64_t>, size_t> by_shape;
    for (size_t i = 0; i < n; ++i) {
        const p3g_trace& t = traces[i];
        const uint64_t work = (uint64_t(1) << (t.log_h + t.log_blowup)) * t.width;
        const bool batch = t.width > 0 && t.log_h >= 1 && t.log_h <= 21;
        if (batch) {
            auto key = std::make_tuple(t.log_h, t.log_blowup, t.shift);
            auto it = by_shape.find(key);
            if (it != by_shape.end()) {
                out[it->second].idx.push_back(i);
                out[it->second].work += work;
                continue;
            }
            by_shape[key] = out.size();
        }
        LdeGroup g;
        g.log_h = int(t.log_h);
        g.log_b = int(t.log_blowup);
        g.shift = t.shift;
        g.batched = batch;
        g.idx.push_back(i);
        g.work = work;
        out.push_back(std::move(g));
    }
    return out;
}

void lde_group_prepare(p3g_ctx* ctx, int field, LdeGroup& g, const p3g_trace* traces, cudaStream_t st) {
    if (!g.batched) return;
    const bool bb = field == P3G_BABYBEAR;
    for (int k = 0; k < 3; ++k) {
        const size_t b = bb ? lde_group_table_bytes_bb(g.log_h, g.log_b, k) : lde_group_table_bytes_gl(g.log_h, g.log_b, k);
        g.tab[k] = b ? ctx->alloc(b, st) : nullptr;
    }
    for (size_t i : g.idx) {
        const size_t b = bb ? lde_group_scr_bytes_bb(g.log_h, int(traces[i].width))
                            : lde_group_scr_bytes_gl(g.log_h, int(traces[i].width));
        g.scr.push_back(b ? ctx->alloc(b, st) : nullptr);
    }
    if (bb) lde_group_tables_bb(ctx, g.log_h, g.log_b, g.shift, g.tab, st);
    else lde_group_tables_gl(ctx, g.log_h, g.log_b, g.shift, g.tab, st);
}

void lde_group_run(p3g_ctx* ctx, int field, const LdeGroup& g, const p3g_trace* traces, const void* const* in,
                   void* const* lde, cudaStream_t st) {
    const bool bb = field == P3G_BABYBEAR;
    if (!g.batched) {
        const size_t i = g.idx[0];
        const p3g_trace& t = traces[i];
        if (bb)
            lde_bb(ctx, static_cast<const uint32_t*>(in[i]), int(t.log_h), int(t.width), int(t.log_blowup),
                   uint32_t(t.shift), 1, static_cast<uint32_t*>(lde[i]), st);
        else
            lde_gl(ctx, static_cast<const uint64_t*>(in[i]), int(t.log_h), int(t.width), int(t.log_blowup), t.shift,
                   1, static_cast<uint64_t*>(lde[i]), st);
        return;
    }
    std::vector<const void*> gin;
    std::vector<void*> gout;
    std::vector<uint32_t> gw;
    for (size_t i : g.idx) {
        gin.push_back(in[i]);
        gout.push_back(lde[i]);
        gw.push_back(traces[i].width);
    }
    if (bb)
        lde_group_bb(ctx, g.log_h, g.log_b, gin.data(), g.scr.data(), gout.data(), gw.data(), g.idx.size(), g.tab, st);
    else
        lde_group_gl(ctx, g.log_h, g.log_b, gin.data(), g.scr.data(), gout.data(), gw.data(), g.idx.size(), g.tab, st);
}

void lde_group_release(p3g_ctx* ctx, LdeGroup& g, cudaStream_t st) {
    for (void*& p : g.tab)
        if (p) {
            ctx->release(p, st);
            p = nullptr;
        }
    for (void* p : g.scr)
        if (p) ctx->release(p, st);
    g.scr.clear();
}

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

// Every trace as a group of its own (no batching): each runs lde_bb / lde_gl.
std::vector<LdeGroup> lde_groups_one_each(const std::vector<p3g_trace>& traces) {
    std::vector<LdeGroup> out;
    for (size_t i = 0; i < traces.size(); ++i) {
        LdeGroup g;
        g.idx.push_back(i);
        g.work = (uint64_t(1) << (traces[i].log_h + traces[i].log_blowup)) * traces[i].width;
        out.push_back(std::move(g));
    }
    return out;
}

// Captures the plan's device work with `k` LDE streams into plan->graph/exec;
// `grouped`: the LDEs of each shape group as one batch.
void capture(p3g_ctx* ctx, p3g_plan* plan, int k, bool grouped) {
    const bool hi = plan->host_input;
    // s[0] is the capture origin and runs the tree build; s[k + 1] copies
    // host inputs
    Streams ss(k + 1 + (hi ? 1 : 0));
    cudaStream_t s0 = ss.s[0];
    cudaStream_t cs = hi ? ss.s[k + 1] : nullptr;
    std::vector<cudaEvent_t> copied(hi ? plan->traces.size() + 1 : 0);
    struct EvGuard {
        std::vector<cudaEvent_t>& v;
        ~EvGuard() {
            for (auto e : v)
                if (e) cudaEventDestroy(e);
        }
    } evg{copied};
    for (auto& e : copied) P3G_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    const size_t esz = plan->field == P3G_BABYBEAR ? 4 : 8;
    P3G_CUDA(cudaStreamBeginCapture(s0, cudaStreamCaptureModeRelaxed));
    try {
        P3G_CUDA(cudaEventRecord(ss.e[0], s0));
        for (int i = 1; i <= k + (hi ? 1 : 0); ++i) P3G_CUDA(cudaStreamWaitEvent(ss.s[i], ss.e[0], 0));
        // The LDE units: the shape groups (one batch launch per pass each) or,
        // with grouping off, every trace on its own.  List scheduling: largest
        // unit first onto the least loaded stream.
        const size_t nt = plan->traces.size();
        std::vector<LdeGroup> single;
        if (!grouped) single = lde_groups_one_each(plan->traces);
        const std::vector<LdeGroup>& units = grouped ? plan->groups : single;
        std::vector<size_t> order(units.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return units[a].work > units[b].work; });
        std::vector<const void*> src(nt);
        for (size_t i = 0; i < nt; ++i) src[i] = hi ? plan->d_traces[i] : plan->traces[i].d_trace;
        std::vector<uint64_t> load(k, 0);
        for (size_t u : order) {
            const LdeGroup& g = units[u];
            const int j = int(std::min_element(load.begin(), load.end()) - load.begin());
            load[j] += g.work + 1;
            cudaStream_t st = ss.s[1 + j];
            if (hi) {
                for (size_t i : g.idx) {
                    const auto& t = plan->traces[i];
                    if (t.width == 0) continue;  // nothing to copy (d_trace may be null)
                    P3G_CUDA(cudaMemcpyAsync(plan->d_traces[i], t.d_trace, esz * (size_t(1) << t.log_h) * t.width,
                                             cudaMemcpyHostToDevice, cs));
                }
                P3G_CUDA(cudaEventRecord(copied[g.idx.back()], cs));
                P3G_CUDA(cudaStreamWaitEvent(st, copied[g.idx.back()], 0));
            }
            lde_group_run(ctx, plan->field, g, plan->traces.data(), src.data(), plan->tree.owned.data(), st);
        }
        if (plan->has_fold) {
            const auto& f = plan->fold;
            cudaStream_t fs = ss.s[1 + (k > 1 ? k - 1 : 0)];
            const void* fin = f.d_in;
            if (hi) {
                P3G_CUDA(cudaMemcpyAsync(plan->d_fold_in, f.d_in, size_t(16) << f.log_height, cudaMemcpyHostToDevice,
                                         cs));
                P3G_CUDA(cudaEventRecord(copied.back(), cs));
                P3G_CUDA(cudaStreamWaitEvent(fs, copied.back(), 0));
                fin = plan->d_fold_in;
            }
            fold_bb4(ctx, static_cast<const uint32_t*>(fin), int(f.log_height), int(f.log_arity), f.beta,
                     static_cast<uint32_t*>(f.d_out), fs);
        }
        for (int i = 1; i <= k + (hi ? 1 : 0); ++i) {
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
    plan->grouped = grouped;
}

// The fastest of `reps` launches after a warm one (the minimum: host-input
// plans see occasional host-to-device copy stalls that have nothing to do
// with the candidate).
float time_launches(p3g_plan* plan, int reps) {
    cudaStream_t st;
    P3G_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    std::vector<cudaEvent_t> ev(reps + 1);
    for (auto& e : ev) P3G_CUDA(cudaEventCreate(&e));
    P3G_CUDA(cudaGraphLaunch(plan->exec, st));  // warm
    P3G_CUDA(cudaEventRecord(ev[0], st));
    for (int i = 0; i < reps; ++i) {
        P3G_CUDA(cudaGraphLaunch(plan->exec, st));
        P3G_CUDA(cudaEventRecord(ev[i + 1], st));
    }
    P3G_CUDA(cudaEventSynchronize(ev[reps]));
    float best = 1e30f;
    for (int i = 0; i < reps; ++i) {
        float ms = 0;
        P3G_CUDA(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
        best = std::min(best, ms);
    }
    for (auto e : ev) cudaEventDestroy(e);
    cudaStreamDestroy(st);
    return best;
}

// --------------------------------------------------------------- autotuner
// Coordinate search, each candidate captured and timed (the fastest of three
// launches):
// first the LDE stage (1, 2, 4 or 8 streams x shape-group batches or one
// launch sequence per trace, which must be more than 1% faster to be taken)
// with the default tree fusion, then the tree's
// layer fusion (the node counts below which levels run cooperatively and
// fuse into one tail CTA).  Leaves the plan captured with the best choice.
// When P3G_TUNE_LOG names a file, every candidate's time is appended to it.
void tune(p3g_ctx* ctx, p3g_plan* plan, const std::string& key) {
    const char* log_path = std::getenv("P3G_TUNE_LOG");
    std::ofstream log;
    if (log_path) log.open(log_path, std::ios::app);
    auto note = [&](int k, bool g, uint64_t tail, uint64_t coop, float ms) {
        if (log.is_open())
            log << key << " streams=" << k << " grouped=" << g << " tail=" << tail << " coop=" << coop << " ms=" << ms
                << "\n";
    };
    const int nt = int(plan->traces.size());
    int best_k = 1;
    bool best_g = true;
    float best_ms = 1e30f;
    for (int gr = 1; gr >= 0; --gr)
        for (int k : {1, 2, 4, 8}) {
            if (k > nt && k > 1) break;
            capture(ctx, plan, k, gr != 0);
            const float ms = time_launches(plan, 3);
            note(k, gr != 0, 0, 0, ms);
            // per-trace launch sequences must win by more than 1%: otherwise
            // the shape-group batches (far fewer graph nodes) are kept
            if (ms < (gr ? 1.0f : 0.99f) * best_ms) {
                best_ms = ms;
                best_k = k;
                best_g = gr != 0;
            }
        }
    const bool bb = plan->field == P3G_BABYBEAR;
    uint64_t best_t = 0, best_c = 0;  // the defaults were timed above
    const std::vector<std::pair<uint64_t, uint64_t>> fusion =
        bb ? std::vector<std::pair<uint64_t, uint64_t>>{{64, 2048}, {256, 8192}, {1024, 8192}, {64, 32768}, {256, 32768}}
           : std::vector<std::pair<uint64_t, uint64_t>>{{64, 0}, {128, 0}};
    for (const auto& f : fusion) {
        plan->tree.tail_max = f.first;
        plan->tree.coop_max = f.second;
        capture(ctx, plan, best_k, best_g);
        const float ms = time_launches(plan, 3);
        note(best_k, best_g, f.first, f.second, ms);
        if (ms < best_ms) {
            best_ms = ms;
            best_t = f.first;
            best_c = f.second;
        }
    }
    plan->tree.tail_max = best_t;
    plan->tree.coop_max = best_c;
    capture(ctx, plan, best_k, best_g);
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
    k << "commit/f" << plan->field << "/n" << plan->traces.size() << "/e2^" << lg << (plan->has_fold ? "/fold" : "")
      << (plan->host_input ? "/host" : "");
    return k.str();
}

// True when `p` is page-locked host memory (allocated or registered with CUDA).
bool is_pinned_host(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

void plan_release(p3g_ctx* ctx, p3g_plan* plan, cudaStream_t st) {
    p3g::tree_release(ctx, &plan->tree, st);
    for (auto& g : plan->groups) lde_group_release(ctx, g, st);
    plan->groups.clear();
    for (void* p : plan->d_traces)
        if (p) ctx->release(p, st);
    plan->d_traces.clear();
    if (plan->d_fold_in) ctx->release(plan->d_fold_in, st);
    plan->d_fold_in = nullptr;
}

int plan_commit(p3g_ctx* ctx, int field, const p3g_trace* traces, size_t n_traces, uint32_t cap_height,
                const p3g_fold_job* fold, uint32_t n_streams, bool host_input, p3g_plan** out) {
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
        plan->host_input = host_input;
        if (fold) {
            plan->has_fold = true;
            plan->fold = *fold;
            P3G_REQUIRE(fold->d_in && fold->d_out, "plan_commit: null fold buffer");
            P3G_REQUIRE(!host_input || is_pinned_host(fold->d_in),
                        "plan_commit_host: the fold input must be pinned host memory");
        }
        const size_t esz = field == P3G_BABYBEAR ? 4 : 8;
        cudaStream_t st0 = nullptr;
        try {
            for (const auto& t : plan->traces) {
                P3G_REQUIRE(t.width == 0 || t.d_trace, "plan_commit: null trace");
                P3G_REQUIRE(t.log_h + t.log_blowup <= (field == P3G_BABYBEAR ? 27u : 32u),
                            "plan_commit: log_h + log_blowup exceeds two-adicity");
                const uint64_t fp = field == P3G_BABYBEAR ? uint64_t(p3g::bb::P) : p3g::gl::P;
                P3G_REQUIRE(t.shift < fp && t.shift != 0, "plan_commit: shift must be canonical and non-zero");
                if (t.log_h > 26) throw p3g::Error(P3G_EUNSUPPORTED, "plan_commit: log_h > 26 is not supported");
                const uint64_t H = uint64_t(1) << (t.log_h + t.log_blowup);
                void* lde = ctx->alloc(esz * H * std::max<uint32_t>(t.width, 1), st0);
                plan->tree.owned.push_back(lde);
                plan->tree.mats.push_back(p3g_matrix{lde, H, t.width, 0});
                if (host_input) {
                    P3G_REQUIRE(t.width == 0 || is_pinned_host(t.d_trace),
                                "plan_commit_host: traces must be pinned host memory");
                    plan->d_traces.push_back(ctx->alloc(esz * (size_t(1) << t.log_h) * std::max<uint32_t>(t.width, 1),
                                                        st0));
                }
            }
            if (host_input && fold) plan->d_fold_in = ctx->alloc(size_t(16) << fold->log_height, st0);
            p3g::tree_prepare(ctx, &plan->tree, cap_height, false, st0, true);
            // LDE shape groups: tables filled and scratch allocated once, here
            plan->groups = p3g::lde_groups(plan->traces.data(), plan->traces.size());
            for (auto& g : plan->groups) p3g::lde_group_prepare(ctx, field, g, plan->traces.data(), st0);
            P3G_CUDA(cudaStreamSynchronize(st0));
            if (n_streams > 0) {
                p3g::capture(ctx, plan.get(), int(n_streams), true);
            } else {
                std::lock_guard<std::mutex> lk(p3g::g_tune_mu);
                p3g::tune_load();
                const std::string key = p3g::tune_key(plan.get());
                auto ks = p3g::g_tune.find(key + "/streams"), kg = p3g::g_tune.find(key + "/grouped");
                auto kt = p3g::g_tune.find(key + "/tail"), kc = p3g::g_tune.find(key + "/coop");
                if (ks != p3g::g_tune.end() && kg != p3g::g_tune.end() && kt != p3g::g_tune.end() &&
                    kc != p3g::g_tune.end()) {
                    plan->tree.tail_max = uint64_t(kt->second);
                    plan->tree.coop_max = uint64_t(kc->second);
                    p3g::capture(ctx, plan.get(), ks->second, kg->second != 0);
                } else {
                    p3g::tune(ctx, plan.get(), key);
                    p3g::g_tune[key + "/streams"] = plan->nstreams;
                    p3g::g_tune[key + "/grouped"] = plan->grouped ? 1 : 0;
                    p3g::g_tune[key + "/tail"] = int(plan->tree.tail_max);
                    p3g::g_tune[key + "/coop"] = int(plan->tree.coop_max);
                    p3g::tune_store();
                }
            }
            P3G_CUDA(cudaDeviceSynchronize());
        } catch (...) {
            if (plan->exec) cudaGraphExecDestroy(plan->exec);
            if (plan->graph) cudaGraphDestroy(plan->graph);
            p3g::plan_release(ctx, plan.get(), st0);
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

}  // namespace
}  // namespace p3g

extern "C" {

int p3g_plan_commit(p3g_ctx* ctx, int field, const p3g_trace* traces, size_t n_traces, uint32_t cap_height,
                    const p3g_fold_job* fold, uint32_t n_streams, p3g_plan** out) {
    return p3g::plan_commit(ctx, field, traces, n_traces, cap_height, fold, n_streams, false, out);
}

int p3g_plan_commit_host(p3g_ctx* ctx, int field, const p3g_trace* traces, size_t n_traces, uint32_t cap_height,
                         const p3g_fold_job* fold, uint32_t n_streams, p3g_plan** out) {
    return p3g::plan_commit(ctx, field, traces, n_traces, cap_height, fold, n_streams, true, out);
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
        p3g::plan_release(ctx, plan, nullptr);
        P3G_CUDA(cudaDeviceSynchronize());
        delete plan;
    } catch (const p3g::Error& e) {
        p3g::set_last_error(e.what());
        return e.status;
    }
    return P3G_OK;
}

}  // extern "C"
