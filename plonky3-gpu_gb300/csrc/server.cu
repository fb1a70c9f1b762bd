// server.cu -- continuous-batching commit+fold service on one GPU.
//
// Requests (a host-resident BabyBear trace, blowup, shift, fold challenge)
// are queued by any host thread; one worker thread admits the queue head as
// soon as a slot (a CUDA stream) is free AND its device-memory footprint fits
// the budget, so requests that arrive while others run are admitted as slots
// and memory free up and their work overlaps on the device.  Each admitted
// request runs, stream-ordered on its slot: host->device copy of the trace,
// coset LDE with bit-reversed rows (radix2_dit.hpp:221-233 + util.hpp:33-45),
// the Poseidon2 MMCS commit (merkle_tree_mmcs.hpp:100-107), and fold_matrix
// (fri_folding.hpp:200) of the LDE's first four columns read as one
// BabyBear^4 column (a stand-in quotient), then the root and the first
// folded value are copied back.  The LDE, its tree and the folded vector (the
// next FRI round's input) stay resident for follow-up openings
// (MerkleTreeMmcs::open_batch, merkle_tree_mmcs.hpp:120-152) and reads of the
// fold until the client releases the request.  Results carry submit / admit /
// done timestamps for latency percentiles.
//
// All waits are bounded: the worker sleeps on a condition variable with a
// timeout, and completion is detected by polling events, so a stalled
// request never blocks the host indefinitely.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "internal.hpp"

namespace {

using Clock = std::chrono::steady_clock;
inline uint64_t now_ns() {
    return uint64_t(std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now().time_since_epoch()).count());
}

__global__ void k_pack4(const uint32_t* __restrict__ lde, uint32_t w, uint64_t rows, uint4* __restrict__ out) {
    const uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const uint32_t* row = lde + r * w;
    out[r] = make_uint4(row[0], row[1], row[2], row[3]);
}

struct Job {
    p3g_request req;
    uint64_t t_submit = 0, t_admit = 0, t_done = 0;
    uint64_t bytes = 0;
    int status = P3G_OK;
    // device state
    int slot = -1;
    void* d_trace = nullptr;
    void* d_pack = nullptr;
    void* d_fold = nullptr;
    p3g_tree* tree = nullptr;
    uint32_t* h_out = nullptr;  // pinned: root (8) + fold head (4)
};

}  // namespace

struct p3g_server {
    p3g_ctx* ctx = nullptr;
    uint64_t budget = 0;
    uint64_t used = 0;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> done_ev;
    std::vector<std::shared_ptr<Job>> slot_job;
    uint32_t* h_slots = nullptr;  // pinned: 16 words per slot (root, fold head)
    std::deque<std::shared_ptr<Job>> pending;
    std::deque<p3g_result> completed;
    std::map<uint64_t, std::shared_ptr<Job>> resident;
    std::mutex mu;
    std::condition_variable cv;
    std::thread worker;
    std::atomic<bool> stop{false};
    std::string fatal;
};

namespace p3g {
namespace {

uint64_t footprint(const p3g_request& r) {
    const uint64_t h = uint64_t(1) << r.log_h, H = h << r.log_blowup;
    const uint64_t w = r.width;
    // trace + LDE + LDE scratch (h*w; three times that above 2^21 rows: the
    // coefficients, the inner transforms' output and their staging) + digests
    // (2H * 32 B) + descriptors + packed fold input (H * 16 B) + fold output
    // (H/2 * 16 B) + slack
    const uint64_t scratch = (r.log_h > 21 ? 3 : 1) * 4 * h * w;
    return 4 * h * w + 4 * H * w + scratch + 64 * H + 16 * H + 8 * H + (1u << 20);
}

void finish(p3g_server* s, const std::shared_ptr<Job>& j) {
    p3g_result res{};
    res.id = j->req.id;
    res.status = j->status;
    res.t_submit_ns = j->t_submit;
    res.t_admit_ns = j->t_admit;
    res.t_done_ns = j->t_done;
    if (j->status == P3G_OK && j->h_out) {
        for (int i = 0; i < 8; ++i) res.root[i] = j->h_out[i];
        for (int i = 0; i < 4; ++i) res.fold_head[i] = j->h_out[8 + i];
    }
    s->completed.push_back(res);
}

// The request's working buffers (trace copy, packed fold input); with
// `all`, the resident fold output too.
void free_job_device(p3g_server* s, Job& j, cudaStream_t st, bool all) {
    p3g_ctx* ctx = s->ctx;
    if (j.d_trace) ctx->release(j.d_trace, st);
    if (j.d_pack) ctx->release(j.d_pack, st);
    j.d_trace = j.d_pack = nullptr;
    if (all && j.d_fold) {
        ctx->release(j.d_fold, st);
        j.d_fold = nullptr;
    }
}

// Enqueues the request's whole device work on its slot stream.
void launch(p3g_server* s, const std::shared_ptr<Job>& j) {
    p3g_ctx* ctx = s->ctx;
    cudaStream_t st = s->streams[j->slot];
    const p3g_request& r = j->req;
    const uint64_t h = uint64_t(1) << r.log_h, H = h << r.log_blowup;
    j->d_trace = ctx->alloc(4 * h * r.width, st);
    P3G_CUDA(cudaMemcpyAsync(j->d_trace, r.h_trace, 4 * h * r.width, cudaMemcpyHostToDevice, st));
    auto tree = std::make_unique<p3g_tree>();
    tree->field = P3G_BABYBEAR;
    void* lde = ctx->alloc(4 * H * r.width, st);
    tree->owned.push_back(lde);
    tree->mats.push_back(p3g_matrix{lde, H, r.width, 0});
    j->tree = tree.release();
    lde_bb(ctx, static_cast<const uint32_t*>(j->d_trace), int(r.log_h), int(r.width), int(r.log_blowup),
           uint32_t(r.shift), 1, static_cast<uint32_t*>(lde), st);
    mmcs_build(ctx, j->tree, 0, st);
    j->d_pack = ctx->alloc(16 * H, st);
    j->d_fold = ctx->alloc(16 * (H / 2), st);
    k_pack4<<<unsigned((H + 255) / 256), 256, 0, st>>>(static_cast<const uint32_t*>(lde), r.width, H,
                                                       static_cast<uint4*>(j->d_pack));
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
    fold_bb4(ctx, static_cast<const uint32_t*>(j->d_pack), int(r.log_h + r.log_blowup), 1, r.beta,
             static_cast<uint32_t*>(j->d_fold), st);
    const size_t last = j->tree->layer_size.size() - 1;
    P3G_CUDA(cudaMemcpyAsync(j->h_out, static_cast<const uint32_t*>(j->tree->d_digests) + j->tree->layer_off[last] * 8,
                             32, cudaMemcpyDeviceToHost, st));
    P3G_CUDA(cudaMemcpyAsync(j->h_out + 8, j->d_fold, 16, cudaMemcpyDeviceToHost, st));
    P3G_CUDA(cudaEventRecord(s->done_ev[j->slot], st));
}

void worker_loop(p3g_server* s) {
    cudaSetDevice(s->ctx->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (!s->stop) {
        bool progress = false;
        // completions
        for (size_t k = 0; k < s->slot_job.size(); ++k) {
            auto& j = s->slot_job[k];
            if (!j) continue;
            const cudaError_t q = cudaEventQuery(s->done_ev[k]);
            if (q == cudaErrorNotReady) continue;
            j->t_done = now_ns();
            if (q != cudaSuccess) {
                j->status = P3G_ECUDA;
                s->fatal = cudaGetErrorString(q);
            }
            free_job_device(s, *j, s->streams[k], j->status != P3G_OK);
            finish(s, j);  // copies the root and fold head out of the slot's pinned words
            j->h_out = nullptr;
            if (j->status == P3G_OK) {
                s->resident[j->req.id] = j;  // LDE + tree stay for openings
            } else {
                if (j->tree) tree_release(s->ctx, j->tree, s->streams[k]);
                delete j->tree;
                j->tree = nullptr;
                s->used -= j->bytes;
            }
            j.reset();
            progress = true;
        }
        // admissions: queue head first, as soon as a slot and memory are free
        while (!s->pending.empty()) {
            int free_slot = -1;
            for (size_t k = 0; k < s->slot_job.size(); ++k)
                if (!s->slot_job[k]) {
                    free_slot = int(k);
                    break;
                }
            if (free_slot < 0) break;
            auto j = s->pending.front();
            if (j->bytes > s->budget) {  // can never fit
                s->pending.pop_front();
                j->status = P3G_ENOMEM;
                j->t_admit = j->t_done = now_ns();
                finish(s, j);
                progress = true;
                continue;
            }
            if (s->used + j->bytes > s->budget) break;
            s->pending.pop_front();
            j->slot = free_slot;
            j->t_admit = now_ns();
            s->used += j->bytes;
            s->slot_job[free_slot] = j;
            j->h_out = s->h_slots + 16 * free_slot;
            try {
                launch(s, j);
            } catch (const p3g::Error& e) {
                j->status = e.status;
                s->fatal = e.what();
                cudaEventRecord(s->done_ev[free_slot], s->streams[free_slot]);
            } catch (const std::exception& e) {
                j->status = P3G_ECUDA;
                s->fatal = e.what();
                cudaEventRecord(s->done_ev[free_slot], s->streams[free_slot]);
            }
            progress = true;
        }
        if (!progress) s->cv.wait_for(lk, std::chrono::microseconds(50));
    }
}

}  // namespace
}  // namespace p3g

extern "C" {

int p3g_server_create(p3g_ctx* ctx, uint32_t max_slots, uint64_t mem_budget_bytes, p3g_server** out) {
    try {
        P3G_REQUIRE(ctx && out, "server_create: null argument");
        P3G_REQUIRE(max_slots >= 1 && max_slots <= 64, "server_create: 1..64 slots");
        if (!ctx->has_p2bb) throw p3g::Error(P3G_ESTATE, "server_create: BabyBear Poseidon2 constants are not set");
        P3G_CUDA(cudaSetDevice(ctx->device));
        auto s = std::make_unique<p3g_server>();
        s->ctx = ctx;
        if (mem_budget_bytes == 0) {
            size_t fr = 0, tot = 0;
            P3G_CUDA(cudaMemGetInfo(&fr, &tot));
            mem_budget_bytes = uint64_t(fr) / 10 * 8;  // 80% of what is free now
        }
        s->budget = mem_budget_bytes;
        s->streams.resize(max_slots);
        s->done_ev.resize(max_slots);
        s->slot_job.resize(max_slots);
        for (auto& x : s->streams) P3G_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
        for (auto& x : s->done_ev) P3G_CUDA(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
        P3G_CUDA(cudaMallocHost(reinterpret_cast<void**>(&s->h_slots), 64 * max_slots));
        p3g_server* raw = s.get();
        s->worker = std::thread([raw] { p3g::worker_loop(raw); });
        *out = s.release();
    } catch (const p3g::Error& e) {
        p3g::set_last_error(e.what());
        return e.status;
    } catch (const std::exception& e) {
        p3g::set_last_error(e.what());
        return P3G_ECUDA;
    }
    return P3G_OK;
}

int p3g_server_submit(p3g_server* s, const p3g_request* req) {
    try {
        P3G_REQUIRE(s && req, "server_submit: null argument");
        P3G_REQUIRE(req->width >= 4, "server_submit: width must be >= 4 (the fold reads four columns)");
        P3G_REQUIRE(req->h_trace != nullptr, "server_submit: null trace");
        P3G_REQUIRE(req->log_h + req->log_blowup <= 27 && req->log_h <= 26 && req->log_h + req->log_blowup >= 1,
                    "server_submit: unsupported size");
        P3G_REQUIRE(req->shift % p3g::bb::P != 0 && req->shift < p3g::bb::P, "server_submit: bad shift");
        for (int k = 0; k < 4; ++k) P3G_REQUIRE(req->beta[k] < p3g::bb::P, "server_submit: beta must be canonical");
        auto j = std::make_shared<Job>();
        j->req = *req;
        j->t_submit = now_ns();
        j->bytes = p3g::footprint(*req);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->pending.push_back(j);
        }
        s->cv.notify_one();
    } catch (const p3g::Error& e) {
        p3g::set_last_error(e.what());
        return e.status;
    }
    return P3G_OK;
}

int p3g_server_poll(p3g_server* s, p3g_result* out, size_t max_results, size_t* n_out) {
    if (!s || !n_out || (max_results && !out)) {
        p3g::set_last_error("server_poll: null argument");
        return P3G_EINVAL;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    size_t n = 0;
    while (n < max_results && !s->completed.empty()) {
        out[n++] = s->completed.front();
        s->completed.pop_front();
    }
    *n_out = n;
    return P3G_OK;
}

int p3g_server_pending(p3g_server* s, uint64_t* queued, uint64_t* in_flight, uint64_t* resident,
                       uint64_t* bytes_used) {
    if (!s) {
        p3g::set_last_error("server_pending: null server");
        return P3G_EINVAL;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    uint64_t fl = 0;
    for (auto& j : s->slot_job) fl += j ? 1 : 0;
    if (queued) *queued = s->pending.size();
    if (in_flight) *in_flight = fl;
    if (resident) *resident = s->resident.size();
    if (bytes_used) *bytes_used = s->used;
    return P3G_OK;
}

int p3g_server_open(p3g_server* s, uint64_t id, const uint64_t* h_indices, size_t n_queries, void* h_rows,
                    void* h_proof) {
    try {
        P3G_REQUIRE(s, "server_open: null server");
        std::shared_ptr<Job> j;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            auto it = s->resident.find(id);
            P3G_REQUIRE(it != s->resident.end(), "server_open: no resident result with that id");
            j = it->second;
        }
        P3G_CUDA(cudaSetDevice(s->ctx->device));
        p3g::open_batch(s->ctx, j->tree, h_indices, n_queries, h_rows, h_proof, nullptr);
    } catch (const p3g::Error& e) {
        p3g::set_last_error(e.what());
        return e.status;
    }
    return P3G_OK;
}

int p3g_server_read_fold(p3g_server* s, uint64_t id, void* h_out, uint64_t n_values) {
    try {
        P3G_REQUIRE(s && h_out, "server_read_fold: null argument");
        std::shared_ptr<Job> j;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            auto it = s->resident.find(id);
            P3G_REQUIRE(it != s->resident.end(), "server_read_fold: no resident result with that id");
            j = it->second;
        }
        const uint64_t half = (uint64_t(1) << (j->req.log_h + j->req.log_blowup)) / 2;
        P3G_REQUIRE(n_values == half, "server_read_fold: n_values must be half the LDE height");
        P3G_REQUIRE(j->d_fold, "server_read_fold: the fold output is not resident");
        P3G_CUDA(cudaSetDevice(s->ctx->device));
        P3G_CUDA(cudaMemcpy(h_out, j->d_fold, 16 * half, cudaMemcpyDeviceToHost));
    } catch (const p3g::Error& e) {
        p3g::set_last_error(e.what());
        return e.status;
    }
    return P3G_OK;
}

int p3g_server_release(p3g_server* s, uint64_t id) {
    try {
        P3G_REQUIRE(s, "server_release: null server");
        std::shared_ptr<Job> j;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            auto it = s->resident.find(id);
            P3G_REQUIRE(it != s->resident.end(), "server_release: no resident result with that id");
            j = it->second;
            s->resident.erase(it);
        }
        P3G_CUDA(cudaSetDevice(s->ctx->device));
        p3g::tree_release(s->ctx, j->tree, nullptr);
        delete j->tree;
        j->tree = nullptr;
        p3g::free_job_device(s, *j, nullptr, true);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->used -= j->bytes;
        }
        s->cv.notify_one();
    } catch (const p3g::Error& e) {
        p3g::set_last_error(e.what());
        return e.status;
    }
    return P3G_OK;
}

int p3g_server_destroy(p3g_server* s) {
    if (!s) return P3G_OK;
    s->stop = true;
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->ctx->device);
    cudaDeviceSynchronize();
    for (auto& kv : s->resident) {
        p3g::tree_release(s->ctx, kv.second->tree, nullptr);
        delete kv.second->tree;
        p3g::free_job_device(s, *kv.second, nullptr, true);
    }
    for (auto& j : s->slot_job)
        if (j) {
            p3g::free_job_device(s, *j, nullptr, true);
            if (j->tree) p3g::tree_release(s->ctx, j->tree, nullptr);
            delete j->tree;
        }
    cudaDeviceSynchronize();
    if (s->h_slots) cudaFreeHost(s->h_slots);
    for (auto x : s->streams) cudaStreamDestroy(x);
    for (auto x : s->done_ev) cudaEventDestroy(x);
    delete s;
    return P3G_OK;
}

}  // extern "C"
