// Autotuner of the batched launch shapes (no counterpart in the reference).
//
// For one call shape (batch-size bucket, topk, nprobe) it runs the search with
// every candidate shape on the caller's queries, checks that each candidate's
// ids and distances equal those of the built-in shapes (every candidate is an
// exact restatement, so any difference is a defect and the candidate is
// dropped), times each with CUDA events on the caller's stream (best of three
// after a warm-up), and keeps the fastest in the index; later calls of that
// shape, and graphs captured from them, use it.
//
//   exact form   scan mode (CTA per query with the split pass for the largest
//                probes, its CTA scan plain or warp-specialised / split pass
//                for every query / warp per query), the
//                deferral threshold, the split pass's exact prefix and its
//                speculation levels
//   tensor-core  (query, cluster) pairs per MMA chunk (the MMA's N)
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "saqg_internal.h"

namespace saqg {

namespace {

struct DevOut {
    void *ids = nullptr, *d = nullptr;
    size_t n = 0;
    explicit DevOut(size_t count) : n(count) {
        if (cudaMalloc(&ids, 4 * std::max<size_t>(n, 1)) != cudaSuccess ||
            cudaMalloc(&d, 4 * std::max<size_t>(n, 1)) != cudaSuccess) {
            cudaGetLastError();
            release();
            throw Error{SAQG_ERR_NOMEM, "autotune: cudaMalloc of the output buffers failed"};
        }
    }
    void release() {
        if (ids) cudaFree(ids);
        if (d) cudaFree(d);
        ids = d = nullptr;
    }
    ~DevOut() { release(); }
    std::vector<uint32_t> host(bool dist) const {
        std::vector<uint32_t> h(n);
        SAQG_CUDA_TRY(cudaMemcpy(h.data(), dist ? d : ids, 4 * n, cudaMemcpyDeviceToHost));
        return h;
    }
};

struct Events {
    cudaEvent_t a = nullptr, b = nullptr;
    Events() {
        SAQG_CUDA_TRY(cudaEventCreate(&a));
        SAQG_CUDA_TRY(cudaEventCreate(&b));
    }
    ~Events() {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
};

// Best of three timed calls after one warm-up call, in ms.
template <class F>
float time_call(F call, cudaStream_t st, Events &ev) {
    call();
    float best = 1e30f;
    for (int r = 0; r < 3; ++r) {
        SAQG_CUDA_TRY(cudaEventRecord(ev.a, st));
        call();
        SAQG_CUDA_TRY(cudaEventRecord(ev.b, st));
        SAQG_CUDA_TRY(cudaEventSynchronize(ev.b));
        float ms = 0;
        SAQG_CUDA_TRY(cudaEventElapsedTime(&ms, ev.a, ev.b));
        best = std::min(best, ms);
    }
    return best;
}

}  // namespace

TuneReport autotune_exact(const Index &I, const float *q, int64_t nq, int64_t topk, int64_t nprobe, float m,
                          cudaStream_t st) {
    SAQG_REQUIRE(nq >= 1, "autotune needs at least one query");
    std::vector<ScanTune> cands;
    ScanTune dflt;  // built-in
    cands.push_back(dflt);
    for (int defer : {256, 512, 1024, 2048, 4096})
        for (int first : {16, 64}) cands.push_back(ScanTune{0, defer, first, -1});
    for (int lv = 1; lv < 5; ++lv) cands.push_back(ScanTune{0, 1024, 16, lv});  // the speculation level sets
    for (int defer : {-1, 4096}) cands.push_back(ScanTune{3, defer, -1, -1});  // warp-specialised CTA scan
    cands.push_back(ScanTune{1, -1, -1, -1});
    if (topk <= 256) cands.push_back(ScanTune{2, -1, -1, -1});
    DevOut ref((size_t)nq * topk), out((size_t)nq * topk);
    Events ev;
    TuneReport rep;
    std::vector<uint32_t> want_ids, want_d;
    for (size_t i = 0; i < cands.size(); ++i) {
        SearchOpts o;
        o.tune = &cands[i];
        const DevOut &dst = i == 0 ? ref : out;
        const float ms = time_call(
            [&] {
                run_search(I, q, nq, topk, nprobe, m, static_cast<uint32_t *>(dst.ids), static_cast<float *>(dst.d),
                           SAQG_MEM_DEVICE, st, nullptr, nullptr, nullptr, nullptr, nullptr, &o);
            },
            st, ev);
        if (i == 0) {
            want_ids = ref.host(false);
            want_d = ref.host(true);
            rep.default_ms = ms;
            rep.tuned_ms = ms;
            rep.scan = cands[0];
        } else if (out.host(false) != want_ids || out.host(true) != want_d) {
            continue;  // not the same answers: never chosen
        } else if (ms < rep.tuned_ms) {
            rep.tuned_ms = ms;
            rep.scan = cands[i];
        }
        rep.candidates++;
    }
    std::lock_guard<std::mutex> lk(I.tune_mu);
    I.scan_tunes[TuneKey{0, tune_bucket(nq), topk, nprobe}] = rep.scan;
    return rep;
}

TuneReport autotune_tc(const Index &I, const float *q, int64_t nq, int64_t topk, int64_t nprobe, int64_t L, float m,
                       cudaStream_t st) {
    SAQG_REQUIRE(nq >= 1, "autotune needs at least one query");
    std::vector<TcTune> cands{TcTune{-1}, TcTune{16}, TcTune{32}, TcTune{64}, TcTune{128}};
    DevOut ref((size_t)nq * topk), out((size_t)nq * topk);
    Events ev;
    TuneReport rep;
    std::vector<uint32_t> want_ids, want_d;
    for (size_t i = 0; i < cands.size(); ++i) {
        TcOpts o;
        o.tune = &cands[i];
        const DevOut &dst = i == 0 ? ref : out;
        const float ms = time_call(
            [&] {
                run_search_tc(I, q, nq, topk, nprobe, L, m, static_cast<uint32_t *>(dst.ids),
                              static_cast<float *>(dst.d), nullptr, SAQG_MEM_DEVICE, st, nullptr, nullptr, nullptr, &o);
            },
            st, ev);
        if (i == 0) {
            want_ids = ref.host(false);
            want_d = ref.host(true);
            rep.default_ms = ms;
            rep.tuned_ms = ms;
            rep.tc = cands[0];
        } else if (out.host(false) != want_ids || out.host(true) != want_d) {
            continue;
        } else if (ms < rep.tuned_ms) {
            rep.tuned_ms = ms;
            rep.tc = cands[i];
        }
        rep.candidates++;
    }
    std::lock_guard<std::mutex> lk(I.tune_mu);
    I.tc_tunes[TuneKey{1, tune_bucket(nq), topk, nprobe}] = rep.tc;
    return rep;
}

}  // namespace saqg
