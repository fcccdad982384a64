// Serving loop: continuous batching of single queries on one index.
// Batches run the exact form (every answer the reference's) or, by
// configuration, the tensor-core form (saqg_search_tc_batch's path).
//
// Requests (one query each, with its own nprobe and k) queue on the host.  A
// dispatcher thread forms a batch from everything pending whenever one of the
// `max_inflight` slots is free, and launches it on that slot's stream: the
// query upload, the batched search (saqg_search_batch's path on the slot's own
// search context) and the result download.  So a batch is admitted while the
// previous ones still run, and their work overlaps on the device.  Admission is
// by memory too: a batch is cut until its scratch (computed from its shape)
// fits the budget left by the other in-flight slots.  A completer thread waits
// for each batch's event and hands the rows back to their tickets.  Each
// query's answer is the one the reference returns for it alone.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <thread>
#include <unordered_map>

#include "saqg_internal.h"

namespace saqg {

namespace {

using Clock = std::chrono::steady_clock;

double ms_since(Clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

struct Request {
    uint64_t ticket = 0;
    std::vector<float> q;
    int nprobe = 0, topk = 0;
    Clock::time_point t_submit;
    bool done = false;
    int status = SAQG_OK;
    std::string err;
    std::vector<uint32_t> ids;
    std::vector<float> dists;
    double latency_ms = 0.0;
};

struct Slot {
    SearchCtx ctx;
    cudaStream_t stream = nullptr;
    cudaEvent_t done_ev = nullptr;
    float *h_q = nullptr, *d_q = nullptr, *h_d = nullptr, *d_d = nullptr;
    uint32_t *h_ids = nullptr, *d_ids = nullptr;
    std::vector<int> np, k;
    std::vector<std::shared_ptr<Request>> reqs;
    int kmax = 0;
    bool busy = false;
    int status = SAQG_OK;
    std::string err;
};

}  // namespace

struct Server {
    const Index &I;
    saqg_server_config cfg;
    std::vector<std::unique_ptr<Slot>> slots;
    std::mutex mu;
    std::condition_variable cv_dispatch, cv_complete, cv_result;
    std::deque<std::shared_ptr<Request>> pending;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> tickets;
    std::deque<Slot *> inflight;
    uint64_t next_ticket = 1;
    bool stopping = false, dispatcher_done = false;
    std::thread dispatcher, completer;
    // statistics
    int64_t submitted = 0, completed = 0, batches = 0, shrinks = 0, batched_queries = 0;
    int max_batch_seen = 0, max_inflight_seen = 0;
    std::vector<double> latencies;

    Server(const Index &idx, const saqg_server_config &c) : I(idx), cfg(c) {}

    void run_dispatcher();
    void run_completer();
    void launch(Slot &s);
};

void Server::launch(Slot &s) {
    const int n = (int)s.reqs.size();
    int npmax = 1;
    s.kmax = 1;
    s.np.resize(n);
    s.k.resize(n);
    for (int i = 0; i < n; ++i) {
        std::memcpy(s.h_q + (size_t)i * I.D, s.reqs[i]->q.data(), 4 * (size_t)I.D);
        s.np[i] = s.reqs[i]->nprobe;
        s.k[i] = s.reqs[i]->topk;
        npmax = std::max(npmax, s.np[i]);
        s.kmax = std::max(s.kmax, s.k[i]);
    }
    SAQG_CUDA_TRY(cudaMemcpyAsync(s.d_q, s.h_q, 4 * (size_t)n * I.D, cudaMemcpyHostToDevice, s.stream));
    if (cfg.form == SAQG_FORM_TC) {
        TcOpts o;
        o.ctx = &s.ctx;
        run_search_tc(I, s.d_q, n, s.kmax, npmax, std::max<int64_t>(cfg.shortlist, s.kmax), cfg.searcher_vars_bound_m,
                      s.d_ids, s.d_d, nullptr, SAQG_MEM_DEVICE, s.stream, nullptr, s.np.data(), s.k.data(), &o);
    } else {
        run_search(I, s.d_q, n, s.kmax, npmax, cfg.searcher_vars_bound_m, s.d_ids, s.d_d, SAQG_MEM_DEVICE, s.stream,
                   nullptr, nullptr, s.np.data(), s.k.data(), &s.ctx);
    }
    SAQG_CUDA_TRY(cudaMemcpyAsync(s.h_ids, s.d_ids, 4 * (size_t)n * s.kmax, cudaMemcpyDeviceToHost, s.stream));
    SAQG_CUDA_TRY(cudaMemcpyAsync(s.h_d, s.d_d, 4 * (size_t)n * s.kmax, cudaMemcpyDeviceToHost, s.stream));
    SAQG_CUDA_TRY(cudaEventRecord(s.done_ev, s.stream));
}

void Server::run_dispatcher() {
    cudaSetDevice(I.device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        auto free_slot = [&]() -> Slot * {
            for (auto &s : slots)
                if (!s->busy) return s.get();
            return nullptr;
        };
        cv_dispatch.wait(lk, [&] { return stopping || (!pending.empty() && free_slot()); });
        if (pending.empty() && stopping) break;
        if (pending.empty()) continue;
        // a partial batch waits briefly for more arrivals while other batches run
        if ((int)pending.size() < cfg.max_batch && !inflight.empty() && cfg.max_wait_us > 0 && !stopping) {
            cv_dispatch.wait_for(lk, std::chrono::microseconds(cfg.max_wait_us),
                                 [&] { return stopping || (int)pending.size() >= cfg.max_batch; });
        }
        Slot *s = free_slot();
        if (!s) continue;
        // admission: as many pending queries as fit the batch limit and the memory budget
        int n = std::min<int>((int)pending.size(), cfg.max_batch);
        size_t held = 0;
        for (auto &o : slots)
            if (o.get() != s && o->busy) held += o->ctx.held_bytes();
        int npmax = 1, kmax = 1;
        for (int i = 0; i < n; ++i) {
            npmax = std::max(npmax, pending[i]->nprobe);
            kmax = std::max(kmax, pending[i]->topk);
        }
        while (n > 1 && held + search_bytes_estimate(I, n, kmax, npmax) > (size_t)cfg.mem_budget_bytes) {
            n = (n + 1) / 2;
            ++shrinks;
        }
        s->reqs.assign(pending.begin(), pending.begin() + n);
        pending.erase(pending.begin(), pending.begin() + n);
        s->busy = true;
        s->status = SAQG_OK;
        lk.unlock();
        try {
            launch(*s);
        } catch (const Error &e) {
            s->status = e.code;
            s->err = e.msg;
        } catch (const std::exception &e) {
            s->status = SAQG_ERR_INTERNAL;
            s->err = e.what();
        }
        if (s->status != SAQG_OK) cudaStreamSynchronize(s->stream);  // nothing of the failed batch stays in flight
        lk.lock();
        ++batches;
        batched_queries += n;
        max_batch_seen = std::max(max_batch_seen, n);
        inflight.push_back(s);
        max_inflight_seen = std::max(max_inflight_seen, (int)inflight.size());
        cv_complete.notify_all();
    }
    dispatcher_done = true;
    cv_complete.notify_all();
}

void Server::run_completer() {
    cudaSetDevice(I.device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        cv_complete.wait(lk, [&] { return !inflight.empty() || dispatcher_done; });
        if (inflight.empty()) break;
        Slot *s = inflight.front();
        lk.unlock();
        int status = s->status;
        std::string err = s->err;
        if (status == SAQG_OK) {
            const cudaError_t e = cudaEventSynchronize(s->done_ev);
            if (e != cudaSuccess) {
                status = SAQG_ERR_CUDA;
                err = std::string("batch failed: ") + cudaGetErrorString(e);
            }
        }
        lk.lock();
        for (size_t i = 0; i < s->reqs.size(); ++i) {
            Request &r = *s->reqs[i];
            r.status = status;
            r.err = err;
            if (status == SAQG_OK) {
                r.ids.assign(s->h_ids + i * s->kmax, s->h_ids + i * s->kmax + r.topk);
                r.dists.assign(s->h_d + i * s->kmax, s->h_d + i * s->kmax + r.topk);
            }
            r.latency_ms = ms_since(r.t_submit);
            r.done = true;
            latencies.push_back(r.latency_ms);
            ++completed;
        }
        s->reqs.clear();
        s->busy = false;
        inflight.pop_front();
        cv_result.notify_all();
        cv_dispatch.notify_all();
    }
}

Server *server_create(const Index &I, const saqg_server_config *c) {
    saqg_server_config cfg{};
    if (c) cfg = *c;
    if (cfg.max_batch <= 0) cfg.max_batch = 4096;
    if (cfg.max_inflight <= 0) cfg.max_inflight = 2;
    if (cfg.max_topk <= 0) cfg.max_topk = 100;
    if (cfg.max_nprobe <= 0) cfg.max_nprobe = (int)std::min<int64_t>(256, I.K);
    if (cfg.max_wait_us < 0) cfg.max_wait_us = 0;
    if (cfg.searcher_vars_bound_m <= 0.0f) cfg.searcher_vars_bound_m = 4.0f;
    SAQG_REQUIRE(cfg.form == SAQG_FORM_EXACT || cfg.form == SAQG_FORM_TC, "unknown search form");
    if (cfg.form == SAQG_FORM_TC) {
        if (cfg.shortlist <= 0) cfg.shortlist = std::min(1024, 8 * cfg.max_topk);
        SAQG_REQUIRE(cfg.max_topk <= 1024 && cfg.shortlist >= cfg.max_topk && cfg.shortlist <= 1024,
                     "tensor-core serving: max_topk <= shortlist <= 1024");
        SAQG_REQUIRE(cfg.max_batch <= 8192, "tensor-core serving: at most 8192 queries per batch");
    }
    SAQG_REQUIRE(cfg.max_topk <= 4096 && cfg.max_nprobe <= I.K, "server bounds beyond the index");
    SAQG_REQUIRE(cfg.max_inflight <= 16, "at most 16 batches in flight");
    int prev = 0;
    SAQG_CUDA_TRY(cudaGetDevice(&prev));
    if (prev != I.device) SAQG_CUDA_TRY(cudaSetDevice(I.device));
    if (cfg.mem_budget_bytes <= 0) {
        size_t fr = 0, tot = 0;
        SAQG_CUDA_TRY(cudaMemGetInfo(&fr, &tot));
        cfg.mem_budget_bytes = (int64_t)(fr / 2);
    }
    auto sv = std::make_unique<Server>(I, cfg);
    for (int i = 0; i < cfg.max_inflight; ++i) {
        auto s = std::make_unique<Slot>();
        SAQG_CUDA_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        SAQG_CUDA_TRY(cudaEventCreateWithFlags(&s->done_ev, cudaEventDisableTiming));
        const size_t nq = cfg.max_batch, qb = 4 * nq * I.D, rb = 4 * nq * cfg.max_topk;
        SAQG_CUDA_TRY(cudaMallocHost(&s->h_q, qb));
        SAQG_CUDA_TRY(cudaMallocHost(&s->h_ids, rb));
        SAQG_CUDA_TRY(cudaMallocHost(&s->h_d, rb));
        SAQG_CUDA_TRY(cudaMalloc(&s->d_q, qb));
        SAQG_CUDA_TRY(cudaMalloc(&s->d_ids, rb));
        SAQG_CUDA_TRY(cudaMalloc(&s->d_d, rb));
        // arenas sized once for the largest batch the budget admits
        int64_t n = cfg.max_batch;
        while (n > 1 && search_bytes_estimate(I, n, cfg.max_topk, cfg.max_nprobe) * cfg.max_inflight >
                            (size_t)cfg.mem_budget_bytes)
            n = (n + 1) / 2;
        if (cfg.form == SAQG_FORM_TC)  // the candidate arena grows with the batches it meets
            presize_tc_ctx(I, s->ctx, n, cfg.max_topk, cfg.max_nprobe, cfg.shortlist, 0);
        else
            presize_ctx(I, s->ctx, n, cfg.max_topk, cfg.max_nprobe);
        sv->slots.push_back(std::move(s));
    }
    if (prev != I.device) cudaSetDevice(prev);
    Server *raw = sv.get();
    raw->dispatcher = std::thread([raw] { raw->run_dispatcher(); });
    raw->completer = std::thread([raw] { raw->run_completer(); });
    return sv.release();
}

void server_free(Server *s) {
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_dispatch.notify_all();
    if (s->dispatcher.joinable()) s->dispatcher.join();
    if (s->completer.joinable()) s->completer.join();
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(s->I.device);
    for (auto &sl : s->slots) {
        if (sl->stream) cudaStreamSynchronize(sl->stream);
        cudaFreeHost(sl->h_q);
        cudaFreeHost(sl->h_ids);
        cudaFreeHost(sl->h_d);
        cudaFree(sl->d_q);
        cudaFree(sl->d_ids);
        cudaFree(sl->d_d);
        if (sl->done_ev) cudaEventDestroy(sl->done_ev);
        if (sl->stream) cudaStreamDestroy(sl->stream);
    }
    s->slots.clear();
    cudaSetDevice(prev);
    delete s;
}

uint64_t server_submit(Server *s, const float *q, int nprobe, int topk) {
    SAQG_REQUIRE(nprobe >= 1 && nprobe <= s->cfg.max_nprobe, "nprobe beyond the server's bound");
    SAQG_REQUIRE(topk >= 1 && topk <= s->cfg.max_topk, "topk beyond the server's bound");
    auto r = std::make_shared<Request>();
    r->q.assign(q, q + s->I.D);
    r->nprobe = nprobe;
    r->topk = topk;
    r->t_submit = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    SAQG_REQUIRE(!s->stopping, "server is stopping");
    r->ticket = s->next_ticket++;
    s->tickets[r->ticket] = r;
    s->pending.push_back(r);
    ++s->submitted;
    s->cv_dispatch.notify_one();
    return r->ticket;
}

void server_wait(Server *s, uint64_t ticket, uint32_t *ids, float *dists, double *latency_ms, int timeout_ms) {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    SAQG_REQUIRE(it != s->tickets.end(), "unknown or already collected ticket");
    std::shared_ptr<Request> r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_ms < 0) s->cv_result.wait(lk, ready);
    else if (!s->cv_result.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
        throw Error{SAQG_ERR_TIMEOUT, "result not ready within the timeout"};
    s->tickets.erase(it);
    if (r->status != SAQG_OK) throw Error{r->status, r->err};
    if (ids) std::memcpy(ids, r->ids.data(), 4 * r->ids.size());
    if (dists) std::memcpy(dists, r->dists.data(), 4 * r->dists.size());
    if (latency_ms) *latency_ms = r->latency_ms;
}

void server_stats(Server *s, saqg_server_stats *out) {
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->batches = s->batches;
    out->admission_shrinks = s->shrinks;
    out->max_batch_seen = s->max_batch_seen;
    out->max_inflight_seen = s->max_inflight_seen;
    out->mean_batch = s->batches ? (double)s->batched_queries / (double)s->batches : 0.0;
    if (!s->latencies.empty()) {
        std::vector<double> l = s->latencies;
        auto pct = [&](double p) {
            const size_t i = std::min(l.size() - 1, (size_t)(p * (double)(l.size() - 1) + 0.5));
            std::nth_element(l.begin(), l.begin() + (long)i, l.end());
            return l[i];
        };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
    }
}

// Submits n queries at the given arrival times (seconds from the call) from
// this thread and collects every answer: the open-loop load of a serving
// benchmark, free of any interpreter between arrivals.
void server_run_trace(Server *s, const float *queries, int64_t n, const double *arrival_s, const int *nprobe,
                      const int *topk, int row, uint32_t *ids, float *dists, double *latency_ms) {
    std::vector<uint64_t> t(n);
    const auto t0 = Clock::now();
    for (int64_t i = 0; i < n; ++i) {
        const auto due = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(arrival_s[i]));
        while (Clock::now() < due) {
            const auto left = due - Clock::now();
            if (left > std::chrono::microseconds(200)) std::this_thread::sleep_for(left - std::chrono::microseconds(100));
        }
        t[i] = server_submit(s, queries + (size_t)i * s->I.D, nprobe[i], topk[i]);
    }
    for (int64_t i = 0; i < n; ++i)
        server_wait(s, t[i], ids ? ids + (size_t)i * row : nullptr, dists ? dists + (size_t)i * row : nullptr,
                    latency_ms ? latency_ms + i : nullptr, -1);
}

}  // namespace saqg
