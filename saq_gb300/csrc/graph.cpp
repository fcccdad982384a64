// A batched search of a fixed shape captured into a CUDA graph: its own
// search context is sized once, a warm-up call builds whatever is built lazily
// (centroid norms, kernel attributes, the BLAS handle and workspace), and the
// second call is captured on a private stream.  Each launch then replays all of the
// search's kernels and copies with one call, on the caller's buffers bound at
// capture time (queries updated in place between launches).
#include <memory>

#include "saqg_internal.h"

namespace saqg {

struct SearchGraph {
    const Index &I;
    SearchCtx ctx;
    cudaStream_t cap = nullptr;  // private stream of the warm-up and the capture
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    explicit SearchGraph(const Index &idx) : I(idx) {}
    ~SearchGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (cap) cudaStreamDestroy(cap);
    }
};

SearchGraph *graph_create(const Index &I, int64_t nq, int64_t topk, int64_t nprobe, float m, const float *q_dev,
                          uint32_t *ids_dev, float *dists_dev, cudaStream_t st) {
    SAQG_REQUIRE(nq >= 1, "a graph needs at least one query");
    auto g = std::make_unique<SearchGraph>(I);
    presize_ctx(I, g->ctx, nq, topk, nprobe);
    // the caller's work on the buffers comes first; the legacy stream cannot be captured
    SAQG_CUDA_TRY(cudaStreamSynchronize(st));
    SAQG_CUDA_TRY(cudaStreamCreateWithFlags(&g->cap, cudaStreamNonBlocking));
    st = g->cap;
    // warm-up: everything built on first use happens outside the capture
    run_search(I, q_dev, nq, topk, nprobe, m, ids_dev, dists_dev, SAQG_MEM_DEVICE, st, nullptr, nullptr, nullptr,
               nullptr, &g->ctx);
    SAQG_CUDA_TRY(cudaStreamSynchronize(st));
    SAQG_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
        run_search(I, q_dev, nq, topk, nprobe, m, ids_dev, dists_dev, SAQG_MEM_DEVICE, st, nullptr, nullptr, nullptr,
                   nullptr, &g->ctx);
    } catch (...) {
        cudaGraph_t broken = nullptr;
        cudaStreamEndCapture(st, &broken);
        if (broken) cudaGraphDestroy(broken);
        cudaGetLastError();
        throw;
    }
    SAQG_CUDA_TRY(cudaStreamEndCapture(st, &g->graph));
    SAQG_CUDA_TRY(cudaGraphInstantiate(&g->exec, g->graph, 0));
    return g.release();
}

void graph_launch(SearchGraph *g, cudaStream_t st) { SAQG_CUDA_TRY(cudaGraphLaunch(g->exec, st)); }

void graph_free(SearchGraph *g) { delete g; }

}  // namespace saqg
