// Internal host-side definitions shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/saqg.h"

namespace saqg {

constexpr int kBlock = 32;     // vectors per FastScan block (defines.hpp KFastScanSize)
constexpr int kMaxSeg = 16;    // segments per index
constexpr int kMaxBits = 13;   // KMaxQuantizeBits (defines.hpp)

// ---------------------------------------------------------------- errors
void set_error(const std::string &msg);
struct Error {
    int code;
    std::string msg;
};
#define SAQG_CUDA_TRY(expr)                                                                           \
    do {                                                                                              \
        cudaError_t e__ = (expr);                                                                     \
        if (e__ != cudaSuccess)                                                                       \
            throw ::saqg::Error{SAQG_ERR_CUDA, std::string(#expr " failed: ") + cudaGetErrorString(e__)}; \
    } while (0)
#define SAQG_REQUIRE(cond, msg)                                         \
    do {                                                                \
        if (!(cond)) throw ::saqg::Error{SAQG_ERR_INVALID, (msg)};      \
    } while (0)

void count_launch(int n = 1);

// ---------------------------------------------------------------- device layout
// One segment of the plan, laid out for the GPU.  All clusters are
// concatenated: cluster c owns blocks [blk_off[c], blk_off[c] + nb_c) and
// vectors [vec_off[c], vec_off[c] + n_c).
//
//   codes  : [block][dim/64][32 lanes] of 8 bytes -- the vector's own 1-bit
//            code (MSB-first per 8 dims, as ClusterPacker::pack_short_codes
//            writes it before FastScan packing), interleaved so that lane v of
//            a warp reads vector v of the block with one coalesced 8-byte load.
//   onorm  : [block][32] |o| (including the file's tail lanes)
//   ipcent : [block][32] ip_cent_oa
//   lcode  : [vector][lstride] ex-code in the reference's compacted layout,
//            row padded to 16 bytes
//   exfac  : [vector] (rescale, error)
//   cent   : [cluster][dim] rotated centroid
struct SegDev {
    int dim = 0, bits = 0, pv = 0, lstride = 0, qoff = 0;
    float *P = nullptr;
    uint2 *codes = nullptr;
    float *onorm = nullptr;
    float *ipcent = nullptr;
    uint8_t *lcode = nullptr;
    float2 *exfac = nullptr;
    float *cent = nullptr;
    float c2 = 0.0f;  // compFastIP's (4 / 0.8) * (1 / sqrt(dim)), fixed per segment
};

struct DevIndexView {  // passed to kernels by value
    int S = 0;
    int K = 0;
    int D = 0;       // original dimension
    int Dtot = 0;    // sum of segment dims (padded)
    const float *centroids = nullptr;  // [K][D]
    const float *var = nullptr;        // [Dtot] (zero beyond the stored variance)
    const uint32_t *ids = nullptr;     // [N]
    const int64_t *blk_off = nullptr;  // [K+1]
    const int64_t *vec_off = nullptr;  // [K+1]
    SegDev seg[kMaxSeg];
};

// What one in-flight search owns: scratch arenas and the auxiliary stream of
// the split pass with its fork / join events.  Searches on
// different contexts may run concurrently on different streams.
struct SearchCtx {
    std::mutex mu;
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    void *split_scratch = nullptr;
    size_t split_scratch_bytes = 0;
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // the query preparation's stream (lowest priority: it has slack beside the
    // centroid ranking) with its own fork / join events
    cudaStream_t low = nullptr;
    cudaEvent_t ev_qfork = nullptr, ev_qjoin = nullptr;
    // pooled contexts: the stream of the last call and an event recorded at its
    // end, so a call on another stream waits for that work before reusing the arenas
    cudaStream_t last_stream = nullptr;
    cudaEvent_t ev_done = nullptr;
    bool used = false;
    SearchCtx() = default;
    SearchCtx(const SearchCtx &) = delete;
    SearchCtx &operator=(const SearchCtx &) = delete;
    ~SearchCtx();
    void *scratch_get(size_t bytes);
    void *split_scratch_get(size_t bytes);
    cudaStream_t aux_stream();
    cudaEvent_t fork_event();
    cudaEvent_t join_event();
    cudaStream_t low_stream();
    cudaEvent_t qfork_event();
    cudaEvent_t qjoin_event();
    size_t held_bytes() const { return scratch_bytes + split_scratch_bytes; }
};

// Launch shapes of the exact batched search (values < 0: the built-in choice).
// Every choice returns the same answers; the autotuner picks one per shape.
struct ScanTune {
    int mode = -1;          // 0: CTA per query, split pass for the largest probes; 1: split pass; 2: warp per query;
                            // 3: mode 0 with the warp-specialised CTA scan
    int defer_blocks = -1;  // mode 0: a query probing more blocks than this takes the split pass
    int first_blocks = -1;  // split pass: blocks scanned exactly before the speculation
    int spec_levels = -1;   // mode 0: which set of speculation levels the split pass uses
};
// Launch shape of the tensor-core form: (query, cluster) pairs per MMA chunk
// (the MMA's N; a multiple of 16).  The approximate distances do not depend on it.
struct TcTune {
    int bn = -1;
};
// Key of a tuned shape: (form, batch-size bucket (next power of two), topk, nprobe).
using TuneKey = std::array<int64_t, 4>;
int64_t tune_bucket(int64_t nq);

struct Index {
    // metadata
    int64_t N = 0, D = 0, K = 0;
    uint8_t qcfg_raw[32] = {0};
    std::vector<float> var;  // as stored in the file
    struct SegHost {
        int64_t dim, bits;
        uint8_t cfg_raw[20];
        bool rotated;
        std::vector<float> P;
    };
    std::vector<SegHost> segs;
    bool compact = false;
    std::vector<int64_t> sizes, blk_off, vec_off;
    int64_t total_blocks = 0;
    // device
    DevIndexView view;
    std::vector<void *> allocations;
    int64_t device_bytes = 0;
    int device = 0;
    // search contexts of ordinary calls: a pool that grows with the number of
    // calls in flight at once (each call leases one, see CtxLease)
    mutable std::mutex pool_mu;
    mutable std::vector<std::unique_ptr<SearchCtx>> ctx_pool;
    // probe shortlist: squared centroid norms (built on first use, under init_mu)
    mutable std::mutex init_mu;
    mutable float *cnorm2 = nullptr;
    mutable void *cent_bf16 = nullptr;  // centroids rounded to BF16 (the probe GEMM's operand)
    // tensor-core form: BF16 code matrix [N][Dtot] and the (cluster, tile) list (built on first use, under init_mu)
    mutable void *tc_codes = nullptr;
    mutable void *tc_tiles = nullptr;
    mutable int64_t tc_ntiles = 0;
    // launch shapes chosen by the autotuner (saqg_autotune), by shape
    mutable std::mutex tune_mu;
    mutable std::map<TuneKey, ScanTune> scan_tunes;
    mutable std::map<TuneKey, TcTune> tc_tunes;
    ~Index();
    void *dalloc(size_t bytes);
    void upload(void *dst, const void *src, size_t bytes);
    // most blocks any nprobe clusters can hold (sizes of the largest clusters)
    std::vector<int64_t> top_blocks_prefix;
    int64_t max_blocks_of_probes(int64_t nprobe) const;
};

// index_io.cpp
Index *load_index_file(const std::string &path);
void save_index_file(const Index &idx, const std::string &path);
void finalize_view(Index &idx);
void save_index_v2(const Index &idx, const std::string &path);
// Host-only conversion between the reference format and v2 (either direction;
// the source format is detected).
void convert_index_file(const std::string &src, const std::string &dst, int format);

// A search context leased from an index's pool for one call on `st`: an idle
// context (one last used on `st` first), or a new one.  The context's arenas may
// still be read by the previous call's kernels on another stream, so `st` first
// waits for the event recorded at that call's end; the lease records it again on
// release.  Concurrent calls on one index thus overlap on their own streams.
struct CtxLease {
    SearchCtx *c = nullptr;
    cudaStream_t st = nullptr;
    CtxLease(const Index &I, cudaStream_t stream);
    ~CtxLease();
    CtxLease(const CtxLease &) = delete;
    CtxLease &operator=(const CtxLease &) = delete;
};

// Options of the exact search beyond the reference's arguments.
struct SearchOpts {
    const ScanTune *tune = nullptr;  // launch shapes (null: the index's tuned choice for the shape, else built-in)
    const int *np_dev = nullptr;     // per-query nprobe / topk in device memory (graph launches), each
    const int *k_dev = nullptr;      // clamped to [1, nprobe] / [1, topk]
};

// search.cu
void run_search(const Index &idx, const float *q, int64_t nq, int64_t topk, int64_t nprobe, float m, uint32_t *ids,
                float *dists, int mem, cudaStream_t st, saqg_search_stats *stats = nullptr,
                uint32_t *probes_out = nullptr, const int *np_host = nullptr, const int *k_host = nullptr,
                SearchCtx *ctx = nullptr, const SearchOpts *opts = nullptr);
// Copies of per-query nprobe / topk (device arrays, may be null) clamped to
// [1, np_max] / [1, k_max], into np_out / k_out (device, nq each).
void clamp_shape(const int *np, const int *k, int64_t nq, int np_max, int k_max, int *np_out, int *k_out,
                 cudaStream_t st);
// Scratch bytes a batch of this shape needs (both arenas), for admission by memory.
size_t search_bytes_estimate(const Index &idx, int64_t nq, int64_t topk, int64_t nprobe);
// Grows a context's arenas (and creates its stream, events and BLAS handle)
// for batches up to this shape, so later searches allocate nothing.
void presize_ctx(const Index &idx, SearchCtx &ctx, int64_t nq, int64_t topk, int64_t nprobe);
// saqg_search for device pointers with its scratch in a static device array.
void run_search_static(const Index &idx, const float *q, int64_t nq, int64_t topk, int64_t nprobe, float m,
                       uint32_t *ids, float *dists, cudaStream_t stream);
int64_t run_estimate(const Index &idx, const float *q_host, int64_t nprobe, float m, uint32_t *ids, float *acc,
                     float *fast, float *vars, int64_t cap);

// Tensor-core form (search.cu): centroid ranking + query rotation of a batch,
// and the exact re-rank of its shortlist.
void tc_rank_rotate(const Index &idx, SearchCtx &ctx, const float *q, int64_t nq, int64_t nprobe, const int *qnp,
                    float m, float *dist, void *work, uint32_t *probe, float *qrot, float *prune, uint8_t *full,
                    int *fb_list, int *flags, void *qbf, cudaStream_t st);
size_t tc_probe_work_bytes(const Index &idx, int64_t nq);
void tc_rerank(const Index &idx, const uint32_t *probe, int64_t nq, int64_t nprobe, const float *qrot,
               const float *prune, const int *lp, const int *sl_pos, const float *sl_apx, const int *sl_cnt, int L,
               int64_t topk, const int *qk, int *grp, int *gj, int *ng, float *sl_dist, uint32_t *ids, float *dists,
               float *apx, cudaStream_t st);
// Options of the tensor-core form beyond its arguments.
struct TcOpts {
    const TcTune *tune = nullptr;  // null: the index's tuned choice for the shape, else built-in
    const int *np_dev = nullptr;   // per-query nprobe / topk in device memory, clamped as for the exact search
    const int *k_dev = nullptr;
    // > 0: capacity in approximate distances.  The call then never reads sizes
    // back to the host (it can be captured in a graph); a batch needing more
    // sets bit 2 of the error word and returns no candidates.
    int64_t cand_cap = 0;
    SearchCtx *ctx = nullptr;      // a caller's own context (graphs); null: one leased from the index
    int **err_word = nullptr;      // receives the device address of the call's error word
    int64_t *candidates = nullptr; // receives the call's candidate count (calls without cand_cap)
};
// tc_search.cu
void run_search_tc(const Index &idx, const float *q, int64_t nq, int64_t topk, int64_t nprobe, int64_t shortlist,
                   float m, uint32_t *ids, float *dists, float *approx, int mem, cudaStream_t st,
                   saqg_tc_stats *stats, const int *np_host = nullptr, const int *k_host = nullptr,
                   const TcOpts *opts = nullptr);
// Device scratch bytes of a tensor-core call of this shape with a candidate capacity.
void presize_tc_ctx(const Index &idx, SearchCtx &ctx, int64_t nq, int64_t topk, int64_t nprobe, int64_t shortlist,
                    int64_t cand_cap);

// autotune.cpp: time every candidate launch shape of this call on the device
// (outputs checked equal to the built-in shapes'), keep the fastest in the index.
struct TuneReport {
    ScanTune scan;
    TcTune tc;
    int candidates = 0;
    float default_ms = 0, tuned_ms = 0;
};
TuneReport autotune_exact(const Index &idx, const float *q_dev, int64_t nq, int64_t topk, int64_t nprobe, float m,
                          cudaStream_t st);
TuneReport autotune_tc(const Index &idx, const float *q_dev, int64_t nq, int64_t topk, int64_t nprobe,
                       int64_t shortlist, float m, cudaStream_t st);

// graph.cpp
struct GraphCfg {
    int form = SAQG_FORM_EXACT;
    const int *np_dev = nullptr, *k_dev = nullptr;  // per-query arrays in device memory (bound)
    int64_t shortlist = 0;                          // tensor-core form
    int64_t cand_cap = 0;                           // tensor-core form (0: from the warm-up call)
    int autotune = 0;
};
struct SearchGraph;
SearchGraph *graph_create(const Index &idx, int64_t nq, int64_t topk, int64_t nprobe, float m, const float *q_dev,
                          uint32_t *ids_dev, float *dists_dev, cudaStream_t st, const GraphCfg &cfg);
void graph_launch(SearchGraph *g, cudaStream_t st);
int graph_status(SearchGraph *g, cudaStream_t st);
const TuneReport &graph_tune(const SearchGraph *g);
void graph_free(SearchGraph *g);
// probe_gemm.cu: ip (row-major nq x K) = Q C^T with BF16 operands (row-major,
// nq x D and K x D) and FP32 accumulation on the tensor cores; *err is set
// (device) if a pipeline wait timed out.  to_bf16 rounds n floats to nearest.
void probe_ip_gemm(const void *q_bf16, int64_t nq, const void *cent_bf16, int64_t K, int64_t D, float *ip, int *err,
                   cudaStream_t st);
void to_bf16(const float *x, int64_t n, void *y_bf16, cudaStream_t st);

// serve.cpp
struct Server;
Server *server_create(const Index &idx, const saqg_server_config *cfg);
void server_free(Server *s);
uint64_t server_submit(Server *s, const float *q, int nprobe, int topk);
void server_wait(Server *s, uint64_t ticket, uint32_t *ids, float *dists, double *latency_ms, int timeout_ms);
void server_stats(Server *s, saqg_server_stats *out);
void server_run_trace(Server *s, const float *queries, int64_t n, const double *arrival_s, const int *nprobe,
                      const int *topk, int row, uint32_t *ids, float *dists, double *latency_ms);

// encode.cu
void run_caq_encode(const float *resid, int64_t n, int64_t dim, int bits, const float *cent, int rdlmt, float eps,
                    int32_t *codes, float *facs, int mem, cudaStream_t st);
Index *construct_index(const float *data, int64_t n, int64_t dim, const float *centroids, int64_t k,
                       const uint32_t *cids, const saqg_quantize_config &cfg, const float *variance,
                       const float *rotations, uint64_t seed, int data_mem);

// plan.cpp (host) and plan_gpu.cu (device; the same plans)
std::vector<std::pair<int64_t, int64_t>> make_plan(const float *var, int64_t dpad, float avg_bits, bool seg,
                                                   int eqseg);
std::vector<std::pair<int64_t, int64_t>> make_plan_device(const float *dvar, int64_t dpad, float avg_bits,
                                                          cudaStream_t st);
std::vector<std::pair<int64_t, int64_t>> make_plan_gpu(const float *var, int64_t dpad, float avg_bits, bool seg,
                                                       int eqseg, bool var_on_device, cudaStream_t st);

}  // namespace saqg
