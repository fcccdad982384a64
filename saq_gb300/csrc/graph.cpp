// A batched search of a fixed shape captured into a CUDA graph: its own
// search context is sized once, a warm-up call builds whatever is built lazily
// (centroid norms, kernel attributes, the BLAS handle and workspace, the
// tensor-core code matrix), and the next call is captured on a private stream.
// Each launch then replays all of the search's kernels and copies with one
// call, on the caller's buffers bound at capture time (queries, and per-query
// nprobe / topk arrays when given, updated in place between launches).
//
// Either form can be captured.  The exact form never reads sizes back to the
// host.  The tensor-core form is captured with a fixed capacity of approximate
// distances (no host round trip); a launch whose batch needs more reports it
// through the graph's status word instead of writing past the arrays.
#include <algorithm>
#include <memory>

#include "saqg_internal.h"

namespace saqg {

struct SearchGraph {
    const Index &I;
    SearchCtx ctx;
    cudaStream_t cap = nullptr;  // private stream of the warm-up and the capture
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int *err = nullptr;          // tensor-core form: the launch's error word (device)
    TuneReport tune;
    int64_t cand_cap = 0;
    explicit SearchGraph(const Index &idx) : I(idx) {}
    ~SearchGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (cap) cudaStreamDestroy(cap);
    }
};

SearchGraph *graph_create(const Index &I, int64_t nq, int64_t topk, int64_t nprobe, float m, const float *q_dev,
                          uint32_t *ids_dev, float *dists_dev, cudaStream_t st, const GraphCfg &gc) {
    SAQG_REQUIRE(nq >= 1, "a graph needs at least one query");
    SAQG_REQUIRE(gc.form == SAQG_FORM_EXACT || gc.form == SAQG_FORM_TC, "unknown search form");
    auto g = std::make_unique<SearchGraph>(I);
    // the caller's work on the buffers comes first; the legacy stream cannot be captured
    SAQG_CUDA_TRY(cudaStreamSynchronize(st));
    SAQG_CUDA_TRY(cudaStreamCreateWithFlags(&g->cap, cudaStreamNonBlocking));
    st = g->cap;
    auto capture = [&](auto call) {
        call();  // warm-up: everything built on first use happens outside the capture
        SAQG_CUDA_TRY(cudaStreamSynchronize(st));
        SAQG_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            call();
        } catch (...) {
            cudaGraph_t broken = nullptr;
            cudaStreamEndCapture(st, &broken);
            if (broken) cudaGraphDestroy(broken);
            cudaGetLastError();
            throw;
        }
        SAQG_CUDA_TRY(cudaStreamEndCapture(st, &g->graph));
        SAQG_CUDA_TRY(cudaGraphInstantiate(&g->exec, g->graph, 0));
    };
    if (gc.form == SAQG_FORM_EXACT) {
        if (gc.autotune) g->tune = autotune_exact(I, q_dev, nq, topk, nprobe, m, st);
        presize_ctx(I, g->ctx, nq, topk, nprobe);
        SearchOpts o;
        o.np_dev = gc.np_dev;
        o.k_dev = gc.k_dev;
        capture([&] {
            run_search(I, q_dev, nq, topk, nprobe, m, ids_dev, dists_dev, SAQG_MEM_DEVICE, st, nullptr, nullptr,
                       nullptr, nullptr, &g->ctx, &o);
        });
    } else {
        SAQG_REQUIRE(gc.shortlist >= topk, "the shortlist must be at least topk");
        if (gc.autotune) g->tune = autotune_tc(I, q_dev, nq, topk, nprobe, gc.shortlist, m, st);
        // capacity: the caller's, else twice the warm-up batch's candidates (at least one selection chunk per query)
        int64_t cap = gc.cand_cap;
        if (cap <= 0) {
            TcOpts probe_opts;
            probe_opts.np_dev = gc.np_dev;
            probe_opts.k_dev = gc.k_dev;
            probe_opts.ctx = &g->ctx;
            int64_t cands = 0;
            probe_opts.candidates = &cands;
            run_search_tc(I, q_dev, nq, topk, nprobe, gc.shortlist, m, ids_dev, dists_dev, nullptr, SAQG_MEM_DEVICE,
                          st, nullptr, nullptr, nullptr, &probe_opts);
            cap = std::max<int64_t>(2 * cands, 4096 * nq);
        }
        g->cand_cap = cap;
        presize_tc_ctx(I, g->ctx, nq, topk, nprobe, gc.shortlist, cap);
        TcOpts o;
        o.np_dev = gc.np_dev;
        o.k_dev = gc.k_dev;
        o.cand_cap = cap;
        o.ctx = &g->ctx;
        o.err_word = &g->err;
        capture([&] {
            run_search_tc(I, q_dev, nq, topk, nprobe, gc.shortlist, m, ids_dev, dists_dev, nullptr, SAQG_MEM_DEVICE,
                          st, nullptr, nullptr, nullptr, &o);
        });
    }
    return g.release();
}

void graph_launch(SearchGraph *g, cudaStream_t st) { SAQG_CUDA_TRY(cudaGraphLaunch(g->exec, st)); }

// Status of the graph's last launch, read once the launch has completed: the
// error word of the tensor-core form (bit 1: a contraction wait timed out,
// bit 2: the batch needed more approximate distances than the capacity).
int graph_status(SearchGraph *g, cudaStream_t st) {
    if (!g->err) return SAQG_OK;
    int h = 0;
    SAQG_CUDA_TRY(cudaStreamSynchronize(st));
    SAQG_CUDA_TRY(cudaMemcpy(&h, g->err, 4, cudaMemcpyDeviceToHost));
    if (h & 1) throw Error{SAQG_ERR_INTERNAL, "tensor-core contraction: a pipeline wait timed out"};
    if (h & 2) throw Error{SAQG_ERR_NOMEM, "the batch needed more approximate distances than the graph's capacity of " +
                                               std::to_string(g->cand_cap) + "; its results are void"};
    return SAQG_OK;
}

const TuneReport &graph_tune(const SearchGraph *g) { return g->tune; }

void graph_free(SearchGraph *g) { delete g; }

}  // namespace saqg
