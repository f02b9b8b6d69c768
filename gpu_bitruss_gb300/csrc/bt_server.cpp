// bt_server.cpp -- request loop: count / support / decompose jobs on graphs of
// different sizes, admitted against an HBM budget, batched as they arrive.
//
// No reference counterpart: the reference runs one algorithm on one graph per
// process (main.cu:91-128).  The server keeps S slots.  Each slot is a worker
// thread with its own device context and CUDA stream, so the uploads,
// counting kernels and copies of different slots overlap on the GPU.
//
// Admission: a request's device footprint is estimated from its graph (the
// sizes of every array the upload, counting and peeling allocate).  A job
// starts only when a slot is free and its footprint fits in what the budget
// has left.  Requests are taken in arrival order; a request that does not fit
// yet is passed over by later ones that do, at most kMaxSkips times, after
// which admission waits for it.
//
// Continuous batching: when a slot takes a request, every queued request of
// the same kind (supports/counts, msp, exact msp) that also fits joins it, up
// to kBatchEdges edges; requests above kSoloEdges edges run alone.  Together they form one arena (bt_graph_pack layout),
// uploaded once and run by one launch sequence.  A request's result is the
// same alone and in a batch: butterflies never span two graphs of an arena.
//
// One cooperative peeling kernel runs at a time in the process (dev_msp
// serialises them); counting kernels, uploads and copies of other slots run
// beside it.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "bt_internal.h"

namespace {

constexpr uint64_t kBatchEdges = 1ull << 26;  // edges per batched arena, at most
constexpr uint64_t kSoloEdges = 1ull << 22;   // requests above this size run alone
constexpr uint32_t kMaxBatch = 1024;          // requests per batch, at most
constexpr uint32_t kMaxSkips = 64;            // admissions that may pass a waiting request

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// kind of work: requests of one kind share a batch
int kind_of(int op) { return op == BT_OP_BFC || op == BT_OP_EBFC ? 0 : (op == BT_OP_MSP ? 1 : 2); }

struct Request {
    uint64_t id = 0;
    const bt_graph *g = nullptr;
    int op = 0;
    void *out = nullptr;
    uint64_t hub_slots = 0;
    Clock::time_point t_submit, t_admit, t_done;
    bool admitted = false, done = false;
    bt_status status = BT_OK;
    std::string error;
    uint64_t count = 0, support_max = 0;
    uint32_t levels = 0, batch = 1;
    uint32_t skipped = 0;
};

using ReqPtr = std::shared_ptr<Request>;

uint64_t hub_slots_of(const bt_graph *g) {
    uint64_t s = 0;
    for (uint32_t d : g->degrees)
        if (d > 256) {  // bt::kHubMinDeg
            uint64_t sz = 64;
            while (sz < 2ull * d) sz <<= 1;
            s += sz;
        }
    return s;
}

}  // namespace

// Device bytes a job on an arena of these sizes allocates at its peak (every
// array of dev_build_graph, dev_ebfc and dev_msp; CUB temporaries bounded
// above).  count_ctas: resident CTAs of the counting kernel.
uint64_t bt_job_footprint(uint64_t n, uint64_t m, uint64_t hub_slots, uint64_t span, uint64_t count_ctas,
                          bool peel) {
    const uint64_t resident = 36 * m + 24 * n + 8 * hub_slots + (1u << 16);
    const uint64_t upload = 32 * m + 52 * n + (16 * m + 24 * n + (4u << 20));
    const uint64_t count = 8 * span * count_ctas + (1u << 20);
    const uint64_t msp = peel ? 84 * m + 8 * n + (1u << 16) : 0;
    return resident + std::max(upload, count + msp);
}

int dev_count_ctas(bt_ctx *ctx);  // bt_count.cu

extern "C" bt_status bt_job_bytes(bt_ctx *ctx, const bt_graph *const *graphs, uint32_t count, int op,
                                  uint64_t *bytes) {
    if (!ctx || !bytes || (count && !graphs)) return bt_fail(BT_ERR_INVALID, "null argument");
    if (op < BT_OP_BFC || op > BT_OP_MSP_EXACT) return bt_fail(BT_ERR_INVALID, "unknown op");
    uint64_t n = 0, m = 0, hub = 0, span = 0;
    for (uint32_t i = 0; i < count; i++) {
        if (!graphs[i]) return bt_fail(BT_ERR_INVALID, "null graph");
        n += graphs[i]->n;
        m += graphs[i]->m;
        hub += hub_slots_of(graphs[i]);
        span = std::max<uint64_t>(span, graphs[i]->n);
    }
    *bytes = bt_job_footprint(n, m, hub, span, (uint64_t)dev_count_ctas(ctx), kind_of(op) != 0);
    return BT_OK;
}

struct bt_server {
    int device = 0;
    uint64_t budget = 0, reserved = 0;
    uint64_t count_ctas = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<ReqPtr> queue;
    std::unordered_map<uint64_t, ReqPtr> reqs;
    std::vector<std::thread> workers;
    std::vector<bt_ctx *> ctxs;
    bool stop = false;
    uint64_t next_id = 1;
    uint32_t running = 0;
    std::vector<double> latency_ms;  // submit -> done of completed requests
    uint64_t completed = 0, batches = 0, batched_requests = 0;

    uint64_t footprint(const std::vector<ReqPtr> &job) const {
        uint64_t n = 0, m = 0, hub = 0, span = 0;
        for (const auto &r : job) {
            n += r->g->n;
            m += r->g->m;
            hub += r->hub_slots;
            span = std::max<uint64_t>(span, r->g->n);
        }
        return bt_job_footprint(n, m, hub, span, count_ctas, kind_of(job[0]->op) != 0);
    }

    // pick a job (lock held); empty if nothing can start now
    std::vector<ReqPtr> pick() {
        std::vector<ReqPtr> job;
        const uint64_t avail = budget - reserved;
        for (size_t qi = 0; qi < queue.size(); qi++) {
            ReqPtr r = queue[qi];
            const uint64_t need = footprint({r});
            if (need > budget) {  // can never fit: fail it now
                r->status = BT_ERR_DEVICE_MEMORY;
                r->error = "request needs " + std::to_string(need) + " device bytes; the server budget is " +
                           std::to_string(budget);
                r->done = true;
                r->t_admit = r->t_done = Clock::now();
                queue.erase(queue.begin() + (long)qi);
                qi--;
                cv_done.notify_all();
                continue;
            }
            if (need > avail) {
                if (r->skipped >= kMaxSkips) return job;  // admission waits for this one
                continue;
            }
            job.push_back(r);
            // requests passed over on the way
            for (size_t k = 0; k < qi; k++) queue[k]->skipped++;
            queue.erase(queue.begin() + (long)qi);
            // continuous batching: later requests of the same kind that fit.
            // A large request runs alone and small ones never wait behind it:
            // an arena's peel lasts about as long as its largest graph's.
            const int kind = kind_of(r->op);
            uint64_t edges = r->g->m;
            if (edges > kSoloEdges) return job;
            for (size_t k = qi; k < queue.size() && job.size() < kMaxBatch;) {
                ReqPtr q = queue[k];
                if (kind_of(q->op) != kind || q->g->m > kSoloEdges || edges + q->g->m > kBatchEdges) {
                    k++;
                    continue;
                }
                job.push_back(q);
                if (footprint(job) > avail) {
                    job.pop_back();
                    k++;
                    continue;
                }
                edges += q->g->m;
                queue.erase(queue.begin() + (long)k);
            }
            return job;
        }
        return job;
    }

    void run_job(bt_ctx *ctx, std::vector<ReqPtr> &job, uint64_t need);
    void worker(uint32_t slot);
};

void bt_server::run_job(bt_ctx *ctx, std::vector<ReqPtr> &job, uint64_t need) {
    NvtxRange range("bt_server_job");
    const int kind = kind_of(job[0]->op);
    ctx->budget = need;
    ctx->peak = ctx->used;
    bt_status rc = BT_OK;
    std::string err;
    // the arena: one graph as it is, several packed
    std::unique_ptr<bt_graph> packed;
    const bt_graph *arena = job[0]->g;
    if (job.size() > 1) {
        std::vector<const bt_graph *> gs;
        for (auto &r : job) gs.push_back(r->g);
        bt_graph *p = nullptr;
        rc = bt_graph_pack(gs.data(), (uint32_t)gs.size(), &p, nullptr);
        packed.reset(p);
        arena = p;
    }
    if (rc == BT_OK) rc = dev_build_graph(ctx, arena);
    std::vector<uint64_t> sup;
    std::vector<uint32_t> res;
    if (rc == BT_OK) {
        if (kind == 0) {
            uint64_t total = 0;
            const bool per_edge = job.size() > 1 || job[0]->op == BT_OP_EBFC;
            rc = dev_ebfc(ctx, per_edge, &total);
            if (rc == BT_OK && per_edge && arena->m) {
                sup.resize(arena->m);
                cudaError_t e = cudaMemcpyAsync(sup.data(), ctx->sup, 8 * arena->m, cudaMemcpyDeviceToHost,
                                                ctx->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
                if (e != cudaSuccess) rc = bt_cuda_fail(e, "support download", __FILE__, __LINE__);
            }
            if (rc == BT_OK && !per_edge) job[0]->count = total;
        } else {
            uint32_t lv = 0;
            rc = dev_msp(ctx, kind == 2, &lv);
            if (rc == BT_OK && arena->m) {
                res.resize(arena->m);
                cudaError_t e = cudaMemcpyAsync(res.data(), ctx->result, 4 * arena->m, cudaMemcpyDeviceToHost,
                                                ctx->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
                if (e != cudaSuccess) rc = bt_cuda_fail(e, "result download", __FILE__, __LINE__);
            }
        }
    }
    if (rc != BT_OK) err = bt_last_error();
    // split the arena's results per request
    uint64_t e0 = 0;
    for (auto &r : job) {
        const uint64_t gm = r->g->m;
        r->status = rc;
        r->error = err;
        r->batch = (uint32_t)job.size();
        if (rc == BT_OK) {
            if (kind == 0 && !sup.empty()) {
                unsigned __int128 s = 0;
                uint64_t mx = 0;
                for (uint64_t e = 0; e < gm; e++) {
                    s += sup[e0 + e];
                    mx = std::max(mx, sup[e0 + e]);
                }
                r->count = (uint64_t)(s / 4);
                r->support_max = mx;
                if (r->op == BT_OP_EBFC && r->out && gm)
                    std::copy(sup.begin() + (long)e0, sup.begin() + (long)(e0 + gm), (uint64_t *)r->out);
            } else if (kind != 0) {
                uint32_t mx = 0;
                for (uint64_t e = 0; e < gm; e++) mx = std::max(mx, res[e0 + e]);
                r->levels = mx;
                if (r->out && gm) std::copy(res.begin() + (long)e0, res.begin() + (long)(e0 + gm), (uint32_t *)r->out);
            }
        }
        e0 += gm;
    }
    // the slot keeps nothing between jobs: its reservation covers all it holds
    ctx_release_graph(ctx);
    ctx_free(ctx, ctx->scratch);
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
    cudaStreamSynchronize(ctx->stream);
    ctx->budget = 0;
}

void bt_server::worker(uint32_t slot) {
    bt_ctx *ctx = ctxs[slot];
    cudaSetDevice(device);
    for (;;) {
        std::vector<ReqPtr> job;
        uint64_t need = 0;
        {
            std::unique_lock<std::mutex> lk(mu);
            for (;;) {
                if (stop && queue.empty()) return;
                if (!queue.empty()) {
                    job = pick();
                    if (!job.empty()) break;
                }
                cv_work.wait(lk);
            }
            need = footprint(job);
            reserved += need;
            running++;
            const auto now = Clock::now();
            for (auto &r : job) {
                r->admitted = true;
                r->t_admit = now;
            }
            if (job.size() > 1) {
                batches++;
                batched_requests += job.size();
            }
        }
        run_job(ctx, job, need);
        {
            std::lock_guard<std::mutex> lk(mu);
            reserved -= need;
            running--;
            const auto now = Clock::now();
            for (auto &r : job) {
                r->t_done = now;
                r->done = true;
                latency_ms.push_back(ms_between(r->t_submit, now));
                completed++;
            }
        }
        cv_done.notify_all();
        cv_work.notify_all();
    }
}

extern "C" bt_status bt_server_create(int device, uint32_t slots, uint64_t hbm_budget, bt_server **out) {
    if (!out) return bt_fail(BT_ERR_INVALID, "null argument");
    *out = nullptr;
    if (slots == 0 || slots > 64) return bt_fail(BT_ERR_INVALID, "slots must be in [1, 64]");
    std::unique_ptr<bt_server> s(new (std::nothrow) bt_server());
    if (!s) return bt_fail(BT_ERR_HOST_MEMORY, "host allocation failed");
    s->device = device;
    for (uint32_t i = 0; i < slots; i++) {
        bt_ctx *c = nullptr;
        bt_status rc = bt_ctx_create(device, &c);
        if (rc != BT_OK) {
            for (bt_ctx *x : s->ctxs) bt_ctx_free(x);
            return rc;
        }
        // each slot peels on its share of the SMs, so the slots' peels run
        // side by side (bt_ctx_set_peel_ctas)
        c->peel_ctas = std::max<uint32_t>(1u, (uint32_t)c->sm_count / slots);
        s->ctxs.push_back(c);
    }
    if (hbm_budget == 0) {
        size_t fr = 0, tot = 0;
        BT_CUDA(cudaMemGetInfo(&fr, &tot));
        hbm_budget = (uint64_t)(fr * 0.9);
    }
    s->budget = hbm_budget;
    s->count_ctas = (uint64_t)dev_count_ctas(s->ctxs[0]);
    for (uint32_t i = 0; i < slots; i++) s->workers.emplace_back([srv = s.get(), i]() { srv->worker(i); });
    *out = s.release();
    return BT_OK;
}

extern "C" bt_status bt_server_submit(bt_server *s, const bt_graph *g, int op, void *out, uint64_t *ticket) {
    if (!s || !g || !ticket) return bt_fail(BT_ERR_INVALID, "null argument");
    if (op < BT_OP_BFC || op > BT_OP_MSP_EXACT) return bt_fail(BT_ERR_INVALID, "unknown op");
    auto r = std::make_shared<Request>();
    r->g = g;
    r->op = op;
    r->out = out;
    r->hub_slots = hub_slots_of(g);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return bt_fail(BT_ERR_STATE, "server is shutting down");
        r->id = s->next_id++;
        r->t_submit = Clock::now();
        s->reqs[r->id] = r;
        s->queue.push_back(r);
        *ticket = r->id;
    }
    s->cv_work.notify_one();
    return BT_OK;
}

extern "C" bt_status bt_server_wait(bt_server *s, uint64_t ticket, double timeout_ms, bt_request_info *info) {
    if (!s) return bt_fail(BT_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return bt_fail(BT_ERR_INVALID, "unknown ticket " + std::to_string(ticket));
    ReqPtr r = it->second;
    auto ready = [&]() { return r->done; };
    if (timeout_ms < 0) s->cv_done.wait(lk, ready);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready))
        return bt_fail(BT_ERR_TIMEOUT, "request " + std::to_string(ticket) + " not done yet");
    s->reqs.erase(ticket);
    if (info) {
        info->status = r->status;
        info->count = r->count;
        info->support_max = r->support_max;
        info->levels = r->levels;
        info->batch_size = r->batch;
        info->queue_ms = ms_between(r->t_submit, r->t_admit);
        info->run_ms = ms_between(r->t_admit, r->t_done);
        info->total_ms = ms_between(r->t_submit, r->t_done);
    }
    if (r->status != BT_OK) return bt_fail(r->status, r->error);
    return BT_OK;
}

extern "C" bt_status bt_server_latency(bt_server *s, double *p50_ms, double *p99_ms, uint64_t *completed,
                                       int reset) {
    if (!s) return bt_fail(BT_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    std::vector<double> v = s->latency_ms;
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) {
        if (v.empty()) return -1.0;
        size_t i = (size_t)(p * (double)(v.size() - 1) + 0.5);
        return v[std::min(i, v.size() - 1)];
    };
    if (p50_ms) *p50_ms = pct(0.50);
    if (p99_ms) *p99_ms = pct(0.99);
    if (completed) *completed = s->completed;
    if (reset) {
        s->latency_ms.clear();
        s->completed = 0;
    }
    return BT_OK;
}

extern "C" bt_status bt_server_stats(bt_server *s, uint64_t *out, int n) {
    if (!s || !out) return bt_fail(BT_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    const uint64_t v[6] = {s->budget, s->reserved, s->running, s->queue.size(), s->batches, s->batched_requests};
    for (int i = 0; i < n && i < 6; i++) out[i] = v[i];
    return BT_OK;
}

extern "C" void bt_server_free(bt_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->workers) t.join();
    for (bt_ctx *c : s->ctxs) bt_ctx_free(c);
    delete s;
}
