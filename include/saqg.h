/*
 * saqg.h -- C ABI of the GB300-native SAQ search / encode path.
 *
 * Every entry point replaces a call on the reference's header-only C++ API
 * (howarlii/SAQ, saqlib/); the citation beside each one names it.  The ABI uses
 * plain pointers and sizes only: no C++ or torch types cross it, errors are
 * returned as status codes (never thrown), and saqg_last_error() gives the
 * message of the last failure on the calling thread.
 *
 * Memory: pointers named *_host are host memory; functions taking a `mem`
 * argument accept either host (SAQG_MEM_HOST: the library stages the copies,
 * host<->device transfers included) or device pointers (SAQG_MEM_DEVICE: the
 * caller's buffers are used in place, nothing is copied).  `stream` is a
 * cudaStream_t passed as void* (NULL = the legacy default stream).
 *
 * Threading: an index handle is read-only after load/construct.  Searches on
 * one handle may be called from many host threads at once (as the reference's
 * drivers call IVF::search from a thread pool): each call leases a scratch
 * context from the handle's pool (the pool grows to the number of calls in
 * flight), and calls on different streams overlap on the device.  A context
 * reused from a call on another stream first makes the new stream wait for
 * that call's end, so no two calls ever share scratch on the device.
 */
#ifndef SAQG_H
#define SAQG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SAQG_OK 0
#define SAQG_ERR_INVALID 1  /* bad argument (sizes, nprobe > K, unsupported dim ...) */
#define SAQG_ERR_IO 2       /* unreadable / truncated / malformed index file */
#define SAQG_ERR_CUDA 3     /* a CUDA runtime call failed */
#define SAQG_ERR_NOMEM 4    /* device or host allocation failed */
#define SAQG_ERR_INTERNAL 5 /* a device-side consistency check failed */
#define SAQG_ERR_TIMEOUT 6  /* a server result was not ready within the timeout */

#define SAQG_MEM_HOST 0
#define SAQG_MEM_DEVICE 1

#define SAQG_FORMAT_REFERENCE 0 /* the reference's .index format (IVF::save) */
#define SAQG_FORMAT_V2 1        /* versioned, checksummed, tile-aligned device layout */

#define SAQG_DIST_L2 1 /* DistType::L2Sqr (defines.hpp); the only type the search supports */

/* QuantizeConfig + QuantSingleConfig (quantization/config.h:12-74), field for field. */
typedef struct saqg_quantize_config {
    float avg_bits;          /* QuantizeConfig::avg_bits */
    int seg_eqseg;           /* QuantizeConfig::seg_eqseg */
    int enable_segmentation; /* QuantizeConfig::enable_segmentation (default 1) */
    int use_compact_layout;  /* QuantizeConfig::use_compact_layout (default 0) */
    int random_rotation;     /* QuantSingleConfig::random_rotation (default 1) */
    int caq_adj_rd_lmt;      /* QuantSingleConfig::caq_adj_rd_lmt (default 6) */
    float caq_adj_eps;       /* QuantSingleConfig::caq_adj_eps (default 1e-8) */
} saqg_quantize_config;

/* SearcherConfig (quantization/config.h:76-79). */
typedef struct saqg_searcher_config {
    float searcher_vars_bound_m; /* default 4 */
    int dist_type;               /* SAQG_DIST_L2 */
} saqg_searcher_config;

typedef struct saqg_index saqg_index;

typedef struct saqg_index_info {
    int64_t num_data, num_dim, num_clusters;
    int32_t num_segments;
    int32_t seg_dim[16];
    int32_t seg_bits[16];
    int64_t device_bytes; /* bytes of device memory held by the index */
} saqg_index_info;

/* ---- library ---------------------------------------------------------- */
int saqg_version(void);
const char *saqg_last_error(void);
/* Number of kernels this library launched on the calling process so far. */
int64_t saqg_kernel_launches(void);

/* ---- index lifecycle -------------------------------------------------- */
/* IVF::load (index/ivf.hpp:230-264): reads the reference's binary .index file
 * and uploads it to the current CUDA device. */
int saqg_index_load(const char *path, saqg_index **out);
/* IVF::save (index/ivf.hpp:197-228): writes the reference's binary format. */
int saqg_index_save(const saqg_index *index, const char *path);

/* No counterpart in the reference: writes the index in format v2 (a
 * versioned header, the device layout as-is with every array at a 4096-byte
 * aligned offset, a 64-bit checksum per array and for the header).
 * saqg_index_load reads either format (detected by the magic "SAQGIDX2"). */
int saqg_index_save_v2(const saqg_index *index, const char *path);

/* Converts an index file between the reference format and v2 on the host,
 * without a GPU (the source format is detected; `format` is
 * SAQG_FORMAT_REFERENCE or SAQG_FORMAT_V2).  A reference -> v2 -> reference
 * round trip reproduces the file byte for byte.  Corrupt v2 files fail with
 * SAQG_ERR_IO (checksum mismatch). */
int saqg_index_convert(const char *src_path, const char *dst_path, int format);
int saqg_index_free(saqg_index *index);
int saqg_index_get_info(const saqg_index *index, saqg_index_info *out);

/* IVF::construct (index/ivf.hpp:130-184) with IVF::set_variance (ivf.hpp:104-107):
 * builds the index on the GPU from `data` (n x dim, row-major), `centroids`
 * (k x dim) and `cluster_ids` (n).  `variance` (dim, may be NULL -> computed
 * from the data as SaqDataMaker::compute_variance does) and `rotations`
 * (concatenated row-major D_s x D_s matrices of the planned segments, may be
 * NULL -> random orthogonal matrices drawn from `seed`; ignored when
 * cfg->random_rotation is 0).  `data` is host or device memory per
 * `data_mem`; every other input is host memory.  Each vector is rotated with
 * the reference's GEMV summation order. */
int saqg_index_construct(const float *data, int64_t n, int64_t dim, const float *centroids, int64_t k,
                         const uint32_t *cluster_ids, const saqg_quantize_config *cfg, const float *variance,
                         const float *rotations, uint64_t seed, int data_mem, saqg_index **out);

/* ---- search ------------------------------------------------------------ */
/* IVF::search<L2Sqr> (index/ivf.hpp:275-311) for `nq` queries (nq x dim), each
 * as an independent call of the reference: probe the `nprobe` nearest
 * centroids, scan them in order with the reference's pruning, keep `topk`.
 * ids: nq x topk (unfilled slots are 0, as ResultPool leaves them);
 * dists: nq x topk estimated distances (may be NULL; FLT_MAX when unfilled). */
int saqg_search(const saqg_index *index, const float *queries, int64_t nq, int64_t topk, int64_t nprobe,
                const saqg_searcher_config *cfg, uint32_t *ids, float *dists, int mem, void *stream);

/* Measurements of one saqg_search_ex call (the counterpart of the reference's
 * QueryRuntimeMetrics, caq_estimator.hpp:21-25, summed over the batch).
 * Kernel times come from CUDA events on the call's stream. */
typedef struct saqg_search_stats {
    float ms_probe;        /* centroid distances + nprobe selection */
    float ms_qprep;        /* prune bounds + query rotation */
    float ms_scan;         /* the cluster scan (FastScan + re-rank + top-k) */
    float ms_total;        /* first to last kernel */
    int64_t probes;        /* (query, cluster) pairs scanned */
    int64_t blocks;        /* 32-vector blocks scanned */
    int64_t vectors;       /* vectors scanned */
    int64_t reranked;      /* vectors whose accurate distance the reference evaluates */
    int64_t speculative;   /* accurate distances evaluated (a superset of `reranked`) */
    int64_t fast_bytes;    /* algorithmic bytes of the scan: 1-bit codes, |o| factors, centroids */
    int64_t rerank_bytes;  /* algorithmic bytes of the re-rank: ex-codes, ex factors, ids */
    float ms_split;        /* the split pass for giant-cluster queries (auxiliary stream; 0 if unused) */
    float ms_split_first;  /* ... its exact prefix scans (the speculation bounds) */
    float ms_split_spec;   /* ... its speculative tile estimates */
    float ms_split_replay; /* ... its sequential replays */
    int64_t probe_exact;   /* exact query-centroid distances evaluated for the probe ranking */
    int64_t probe_full;    /* queries ranked against every centroid exactly (no shortlist) */
    int64_t probe_full_ties; /* ... of which because of equal distances on the shortlist */
} saqg_search_stats;

/* saqg_search plus measurements: `stats` (may be NULL) and `probes` (may be
 * NULL; nq x nprobe probed cluster ids in probe order, memory per `mem`).
 * With stats the call synchronises its stream before returning. */
int saqg_search_ex(const saqg_index *index, const float *queries, int64_t nq, int64_t topk, int64_t nprobe,
                   const saqg_searcher_config *cfg, uint32_t *ids, float *dists, int mem, void *stream,
                   saqg_search_stats *stats, uint32_t *probes);

/* ---- search without allocation ---------------------------------------- */
/* No counterpart in the reference: saqg_search for callers that must not
 * allocate device memory inside a call (a serving loop beside a framework
 * whose caching allocator holds the device memory, where cudaMalloc fails or
 * cudaFree stalls every stream of the device).  The call allocates nothing:
 * its scratch is one static device array of SAQG_STATIC_SCRATCH_BYTES per
 * device.  Queries (nq x dim), ids and dists (nq x topk; dists may be NULL)
 * are device pointers on the index's device; results equal saqg_search's.
 * A call needs nq * (12 * clusters + 4 * nprobe + 4 * padded dim + 4 * segments)
 * bytes (each term rounded up to 16) + 64; larger calls fail with
 * SAQG_ERR_INVALID before any work.  The first call on a device looks up the
 * array's address (cudaGetSymbolAddress) and may make the driver load the
 * kernels: make it before any stream capture.  Every call on a device shares
 * the array, so calls that overlap on the GPU (other streams, other threads)
 * race: order them on one stream.  The array lives in the module of the search
 * kernels: any process that runs a search kernel of this library on a device
 * holds its 16 MiB there until exit, whether or not it calls this entry point
 * (count it in device-memory budgets).  A host pointer, or one on another
 * device, is rejected with SAQG_ERR_INVALID before any work. */
#define SAQG_STATIC_SCRATCH_BYTES (16u << 20)
int saqg_search_static(const saqg_index *index, const float *queries, int64_t nq, int64_t topk, int64_t nprobe,
                       const saqg_searcher_config *cfg, uint32_t *ids, float *dists, void *stream);

/* IVF::search for a batch whose queries carry their own nprobe and topk
 * (each query an independent call of the reference with its own arguments):
 * `nprobe_per_query` / `topk_per_query` are host arrays of nq values (either
 * may be NULL: then `nprobe` / `topk` for every query).  ids / dists rows are
 * max(topk) long; query i's first topk_i entries are its result and the rest
 * id 0 / FLT_MAX.  `stats` may be NULL; other arguments as saqg_search. */
int saqg_search_batch(const saqg_index *index, const float *queries, int64_t nq, const int32_t *nprobe_per_query,
                      const int32_t *topk_per_query, int64_t nprobe, int64_t topk, const saqg_searcher_config *cfg,
                      uint32_t *ids, float *dists, int mem, void *stream, saqg_search_stats *stats);

/* ---- tensor-core form ---------------------------------------------------- */
/* No counterpart in the reference (its search is one query at a time on
 * AVX-512): a batch of queries answered through a dense product on the tensor
 * cores.  Every probed cluster's full CAQ codes (BF16, exact below 2^8) are
 * multiplied with the BF16-rounded residual queries of the queries probing it
 * (FP32 accumulation); the `shortlist` smallest of these approximate distances
 * per query are re-ranked with the exact distance saqg_search computes for a
 * vector, and the topk smallest of those are returned (equal distances: the
 * later-scanned vector first, as ResultPool orders them).  `dists` (may be
 * NULL) are therefore bit-identical to saqg_search's distance for the same id;
 * `approx` (may be NULL) is each returned vector's tensor-core distance.  Ids a
 * query would see through saqg_search but whose approximate distance ranks
 * beyond the shortlist are missed.  Needs every segment coded (bits >= 1),
 * nq <= 8192, topk <= shortlist <= 1024.  The first call on an index builds
 * the code matrix (2 bytes per vector and dimension of device memory). */
typedef struct saqg_tc_stats {
    float ms_probe;      /* centroid ranking + query rotation */
    float ms_pairs;      /* (query, cluster) pairs bucketed by cluster */
    float ms_contract;   /* the tensor-core contraction (k_tc_contract) */
    float ms_select;     /* shortlist selection */
    float ms_rerank;     /* exact re-rank of the shortlist + top-k */
    int64_t pairs;       /* (query, probed cluster) pairs */
    int64_t candidates;  /* approximate distances produced */
    int64_t tiles;       /* 128-vector tiles contracted */
    int64_t flops;       /* 2 * dim * sum over clusters of (queries x vectors) */
    int64_t mma_flops;   /* ... as issued (tiles of 128 vectors, pairs padded to 16) */
    int64_t code_bytes;  /* code bytes of the probed clusters (each read once) */
} saqg_tc_stats;

int saqg_search_tc(const saqg_index *index, const float *queries, int64_t nq, int64_t topk, int64_t nprobe,
                   int64_t shortlist, const saqg_searcher_config *cfg, uint32_t *ids, float *dists, float *approx,
                   int mem, void *stream, saqg_tc_stats *stats);

/* No counterpart in the reference: saqg_search_tc for a batch whose queries
 * carry their own nprobe and topk, host arrays of nq values (either may be
 * NULL: then `nprobe` / `topk` for every query).  Rows of ids / dists / approx
 * are max(topk) long; query i's first topk_i entries are its result and the
 * rest id 0 / FLT_MAX.  Each query's answer equals its saqg_search_tc answer
 * with its own nprobe and topk and the same shortlist (which must be at least
 * the largest topk). */
int saqg_search_tc_batch(const saqg_index *index, const float *queries, int64_t nq, const int32_t *nprobe_per_query,
                         const int32_t *topk_per_query, int64_t nprobe, int64_t topk, int64_t shortlist,
                         const saqg_searcher_config *cfg, uint32_t *ids, float *dists, float *approx, int mem,
                         void *stream, saqg_tc_stats *stats);

/* ---- graph-captured search ---------------------------------------------- */
/* No counterpart in the reference: saqg_search for a fixed shape (nq, topk,
 * nprobe) on device buffers, captured into a CUDA graph.  Creation runs the
 * search twice on `stream` (a warm-up, then the capture), so `queries` must
 * hold valid data; each saqg_search_graph_launch then replays every kernel and
 * copy with one call, reading `queries` and writing `ids` / `dists` (bound at
 * creation; update the queries in place between launches).  Results equal
 * saqg_search's.  Launches of one graph must not overlap. */
typedef struct saqg_search_graph saqg_search_graph;
int saqg_search_graph_create(const saqg_index *index, const float *queries, int64_t nq, int64_t topk, int64_t nprobe,
                             const saqg_searcher_config *cfg, uint32_t *ids, float *dists, void *stream,
                             saqg_search_graph **out);
int saqg_search_graph_launch(saqg_search_graph *graph, void *stream);
int saqg_search_graph_free(saqg_search_graph *graph);

/* No counterpart in the reference.  Launch shapes of the batched search picked
 * by timing (saqg_autotune) and graphs of either form with per-query nprobe /
 * topk (saqg_search_graph_create_ex). */
#define SAQG_FORM_EXACT 0 /* saqg_search: every answer the reference's */
#define SAQG_FORM_TC 1    /* saqg_search_tc: the tensor-core form */

typedef struct saqg_tune_report {
    int form;            /* SAQG_FORM_EXACT or SAQG_FORM_TC */
    int scan_mode;       /* exact: 0 CTA per query (+ split pass for the largest probes), 1 split pass, 2 warp per query,
                            3 as 0 with the warp-specialised CTA scan; -1 built-in */
    int defer_blocks;    /* exact, mode 0: blocks above which a query takes the split pass (-1 built-in) */
    int first_blocks;    /* exact: blocks the split pass scans before speculating (-1 built-in) */
    int pairs_per_chunk; /* tensor-core form: the MMA's N (-1 built-in) */
    int spec_levels;     /* exact, mode 0: the split pass's set of speculation levels (-1 built-in) */
    int candidates;      /* shapes timed (each one's answers checked equal to the built-in shapes') */
    float default_ms;    /* one call with the built-in shapes (best of 3, CUDA events) */
    float tuned_ms;      /* one call with the chosen shapes */
} saqg_tune_report;

/* Times every candidate launch shape of a call (`queries`: nq x dim, device
 * memory, on `stream`) and keeps the fastest in the index: later calls whose
 * batch size rounds up to the same power of two, with the same topk and nprobe,
 * use it.  `shortlist` is read for SAQG_FORM_TC only.  Allocates and synchronises;
 * call it outside any stream capture. */
int saqg_autotune(const saqg_index *index, const float *queries, int64_t nq, int64_t topk, int64_t nprobe,
                  int64_t shortlist, int form, const saqg_searcher_config *cfg, void *stream,
                  saqg_tune_report *report);

typedef struct saqg_graph_config {
    int form;                         /* SAQG_FORM_EXACT or SAQG_FORM_TC */
    const int32_t *nprobe_per_query;  /* device, nq values, each clamped to [1, nprobe]; NULL: nprobe for all */
    const int32_t *topk_per_query;    /* device, nq values, each clamped to [1, topk]; NULL: topk for all */
    int64_t shortlist;                /* SAQG_FORM_TC: as saqg_search_tc's (>= topk) */
    int64_t candidate_capacity;       /* SAQG_FORM_TC: approximate distances a launch may hold (0: twice the
                                         creation batch's, at least 4096 per query) */
    int autotune;                     /* 1: saqg_autotune this shape before the capture */
} saqg_graph_config;

/* saqg_search_graph_create for either form, with per-query nprobe / topk read
 * from device arrays at every launch (rows of ids / dists are topk long, padded
 * with id 0 / FLT_MAX past a query's own topk).  The tensor-core form is
 * captured with a fixed candidate capacity and reads nothing back to the host;
 * after a launch has completed, saqg_search_graph_status reports whether it
 * fitted (SAQG_ERR_NOMEM: the batch needed more candidates, its results are
 * void) or a contraction wait timed out (SAQG_ERR_INTERNAL).  `report` (may be
 * NULL) receives the autotuner's choice. */
int saqg_search_graph_create_ex(const saqg_index *index, const float *queries, int64_t nq, int64_t topk,
                                int64_t nprobe, const saqg_searcher_config *cfg, const saqg_graph_config *gcfg,
                                uint32_t *ids, float *dists, void *stream, saqg_search_graph **out,
                                saqg_tune_report *report);
int saqg_search_graph_status(saqg_search_graph *graph, void *stream);

/* ---- serving ----------------------------------------------------------- */
/* No counterpart in the reference (its drivers call IVF::search from a thread
 * pool): a serving loop with continuous batching on one index.  Submitted
 * queries (each with its own nprobe and topk) are batched on the device as
 * slots free up: up to `max_inflight` batches run at once on their own streams
 * and search contexts, so a batch is admitted while earlier ones still run.
 * A batch is also cut down until its scratch fits `mem_budget_bytes` minus what
 * the other in-flight batches hold.  Every answer equals the reference's for
 * that query alone (saqg_search_batch's path). */
typedef struct saqg_server saqg_server;
typedef struct saqg_server_config {
    int32_t max_batch;        /* queries per batch at most (0: 4096) */
    int32_t max_inflight;     /* batches on the device at once (0: 2; at most 16) */
    int32_t max_topk;         /* largest topk a request may ask (0: 100) */
    int32_t max_nprobe;       /* largest nprobe a request may ask (0: min(256, clusters)) */
    int32_t max_wait_us;      /* how long a partial batch waits for arrivals while others run */
    float searcher_vars_bound_m; /* SearcherConfig::searcher_vars_bound_m (0: 4) */
    int64_t mem_budget_bytes; /* device scratch for in-flight batches (0: half the free memory) */
    int32_t form;             /* SAQG_FORM_EXACT (saqg_search_batch: every answer the reference's) or
                                 SAQG_FORM_TC (saqg_search_tc_batch: the tensor-core form) */
    int32_t shortlist;        /* SAQG_FORM_TC: approximate distances re-ranked per query (0: 8 x max_topk,
                                 at most 1024) */
} saqg_server_config;

typedef struct saqg_server_stats {
    int64_t submitted, completed, batches, admission_shrinks;
    int32_t max_batch_seen, max_inflight_seen;
    double mean_batch, p50_ms, p99_ms; /* latency from submit to result ready */
} saqg_server_stats;

int saqg_server_create(const saqg_index *index, const saqg_server_config *cfg, saqg_server **out);
/* Queues one query (host memory, dim floats); returns its ticket. */
int saqg_server_submit(saqg_server *server, const float *query, int32_t nprobe, int32_t topk, uint64_t *ticket);
/* Waits for a ticket's result (timeout_ms < 0: no limit) and copies its topk
 * ids / dists (either may be NULL) and latency; the ticket is then spent. */
int saqg_server_wait(saqg_server *server, uint64_t ticket, uint32_t *ids, float *dists, double *latency_ms,
                     int32_t timeout_ms);
int saqg_server_get_stats(saqg_server *server, saqg_server_stats *out);
/* Open-loop load: submits n queries (n x dim host floats) at `arrival_s`
 * seconds from the call, with their nprobe / topk, and collects every result
 * into rows of `row` entries (ids / dists may be NULL) and latencies. */
int saqg_server_run_trace(saqg_server *server, const float *queries, int64_t n, const double *arrival_s,
                          const int32_t *nprobe, const int32_t *topk, int32_t row, uint32_t *ids, float *dists,
                          double *latency_ms);
/* Drains the queue (every submitted query is answered) and releases the server. */
int saqg_server_free(saqg_server *server);

/* IVF::estimate<L2Sqr> (index/ivf.hpp:313-362) for one query: every vector of
 * the `nprobe` probed clusters, in probe order, with its accurate, fast and
 * variance-bound estimates.  Host outputs of capacity `cap`; *count receives
 * the number of vectors (may exceed cap: then only cap are written). */
int saqg_estimate(const saqg_index *index, const float *query_host, int64_t nprobe, const saqg_searcher_config *cfg,
                  uint32_t *ids, float *acc, float *fast, float *vars, int64_t cap, int64_t *count);

/* ---- encode primitives ------------------------------------------------- */
/* SaqDataMaker::analyze_plan (quantization/saq_data.hpp:119-227): segment bit
 * plan for a padded dimension.  Writes up to `cap` (dim, bits) pairs. */
int saqg_plan(const float *variance_host, int64_t dim_padded, float avg_bits, int enable_segmentation, int seg_eqseg,
              int64_t *dims, int64_t *bits, int cap, int *num_segments);

/* The same plan computed on the GPU (SaqDataMaker::dynamic_programming,
 * saq_data.hpp:147-227, one thread per DP state of a level, in the reference's
 * visit order; the plan equals saqg_plan's).  `variance` is host or device
 * memory per `mem`; runs on `stream` and returns when the plan is known.
 * saqg_index_construct plans this way. */
int saqg_plan_gpu(const float *variance, int64_t dim_padded, float avg_bits, int enable_segmentation, int seg_eqseg,
                  int mem, void *stream, int64_t *dims, int64_t *bits, int cap, int *num_segments);

/* CAQEncoder::encode_and_fac (quantization/caq/caq_encoder.hpp:172-247) for n
 * residual vectors of one segment: codes (n x dim int32) and factors
 * (n x 4: o_l2norm, ip_cent_oa, fac_rescale, fac_error).  `centroid` is the
 * un-rotated centroid used for ip_cent_oa (may be NULL). */
int saqg_caq_encode(const float *resid, int64_t n, int64_t dim, int bits, const float *centroid, int rd_lmt,
                    float eps, int32_t *codes, float *factors, int mem, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SAQG_H */
