// extern "C" entry points (include/saqg.h).  Every call catches its errors and
// turns them into a status code plus a thread-local message.
#include <atomic>
#include <cstring>
#include <string>

#include "saqg_internal.h"

namespace saqg {

namespace {
thread_local std::string g_last_error;
std::atomic<int64_t> g_launches{0};
}  // namespace

void set_error(const std::string &msg) { g_last_error = msg; }
void count_launch(int n) { g_launches += n; }

template <class F>
int guarded(F &&f) {
    try {
        f();
        return SAQG_OK;
    } catch (const Error &e) {
        set_error(e.msg);
        return e.code;
    } catch (const std::bad_alloc &) {
        set_error("host allocation failed");
        return SAQG_ERR_NOMEM;
    } catch (const std::exception &e) {
        set_error(e.what());
        return SAQG_ERR_INTERNAL;
    }
}

}  // namespace saqg

using namespace saqg;

struct saqg_index {
    Index *impl;
};

struct saqg_server {
    Server *impl;
};

struct saqg_search_graph {
    SearchGraph *impl;
};

extern "C" {

int saqg_version(void) { return 1; }

const char *saqg_last_error(void) { return g_last_error.c_str(); }

int64_t saqg_kernel_launches(void) { return g_launches.load(); }

int saqg_index_load(const char *path, saqg_index **out) {
    return guarded([&] {
        SAQG_REQUIRE(path && out, "null argument");
        *out = nullptr;
        Index *I = load_index_file(path);
        *out = new saqg_index{I};
    });
}

int saqg_index_save(const saqg_index *index, const char *path) {
    return guarded([&] {
        SAQG_REQUIRE(index && path, "null argument");
        save_index_file(*index->impl, path);
    });
}

int saqg_index_save_v2(const saqg_index *index, const char *path) {
    return guarded([&] {
        SAQG_REQUIRE(index && path, "null argument");
        save_index_v2(*index->impl, path);
    });
}

int saqg_index_convert(const char *src_path, const char *dst_path, int format) {
    return guarded([&] {
        SAQG_REQUIRE(src_path && dst_path, "null argument");
        SAQG_REQUIRE(format == SAQG_FORMAT_REFERENCE || format == SAQG_FORMAT_V2, "unknown index format");
        convert_index_file(src_path, dst_path, format);
    });
}

int saqg_index_free(saqg_index *index) {
    return guarded([&] {
        if (!index) return;
        delete index->impl;
        delete index;
    });
}

int saqg_index_get_info(const saqg_index *index, saqg_index_info *out) {
    return guarded([&] {
        SAQG_REQUIRE(index && out, "null argument");
        const Index &I = *index->impl;
        std::memset(out, 0, sizeof(*out));
        out->num_data = I.N;
        out->num_dim = I.D;
        out->num_clusters = I.K;
        out->num_segments = (int32_t)I.segs.size();
        for (size_t s = 0; s < I.segs.size() && s < 16; ++s) {
            out->seg_dim[s] = (int32_t)I.segs[s].dim;
            out->seg_bits[s] = (int32_t)I.segs[s].bits;
        }
        out->device_bytes = I.device_bytes;
    });
}

int saqg_index_construct(const float *data, int64_t n, int64_t dim, const float *centroids, int64_t k,
                         const uint32_t *cluster_ids, const saqg_quantize_config *cfg, const float *variance,
                         const float *rotations, uint64_t seed, int data_mem, saqg_index **out) {
    return guarded([&] {
        SAQG_REQUIRE(data && centroids && cluster_ids && cfg && out, "null argument");
        SAQG_REQUIRE(n > 0 && dim > 0 && k > 0, "empty input");
        *out = nullptr;
        SAQG_REQUIRE(data_mem == SAQG_MEM_HOST || data_mem == SAQG_MEM_DEVICE, "bad mem flag");
        Index *I = construct_index(data, n, dim, centroids, k, cluster_ids, *cfg, variance, rotations, seed, data_mem);
        *out = new saqg_index{I};
    });
}

int saqg_search(const saqg_index *index, const float *queries, int64_t nq, int64_t topk, int64_t nprobe,
                const saqg_searcher_config *cfg, uint32_t *ids, float *dists, int mem, void *stream) {
    return guarded([&] {
        SAQG_REQUIRE(index && queries && ids, "null argument");
        SAQG_REQUIRE(mem == SAQG_MEM_HOST || mem == SAQG_MEM_DEVICE, "mem must be SAQG_MEM_HOST or SAQG_MEM_DEVICE");
        const float m = cfg ? cfg->searcher_vars_bound_m : 4.0f;
        SAQG_REQUIRE(!cfg || cfg->dist_type == SAQG_DIST_L2, "only L2 search is supported (the reference's IP search "
                                                              "never inserts a result)");
        run_search(*index->impl, queries, nq, topk, nprobe, m, ids, dists, mem, (cudaStream_t)stream);
    });
}

int saqg_search_ex(const saqg_index *index, const float *queries, int64_t nq, int64_t topk, int64_t nprobe,
                   const saqg_searcher_config *cfg, uint32_t *ids, float *dists, int mem, void *stream,
                   saqg_search_stats *stats, uint32_t *probes) {
    return guarded([&] {
        SAQG_REQUIRE(index && queries && ids, "null argument");
        SAQG_REQUIRE(mem == SAQG_MEM_HOST || mem == SAQG_MEM_DEVICE, "mem must be SAQG_MEM_HOST or SAQG_MEM_DEVICE");
        SAQG_REQUIRE(!cfg || cfg->dist_type == SAQG_DIST_L2, "only L2 search is supported");
        const float m = cfg ? cfg->searcher_vars_bound_m : 4.0f;
        run_search(*index->impl, queries, nq, topk, nprobe, m, ids, dists, mem, (cudaStream_t)stream, stats, probes);
    });
}

int saqg_search_batch(const saqg_index *index, const float *queries, int64_t nq, const int32_t *nprobe_per_query,
                      const int32_t *topk_per_query, int64_t nprobe, int64_t topk, const saqg_searcher_config *cfg,
                      uint32_t *ids, float *dists, int mem, void *stream, saqg_search_stats *stats) {
    return guarded([&] {
        SAQG_REQUIRE(index && queries && ids, "null argument");
        SAQG_REQUIRE(mem == SAQG_MEM_HOST || mem == SAQG_MEM_DEVICE, "mem must be SAQG_MEM_HOST or SAQG_MEM_DEVICE");
        SAQG_REQUIRE(!cfg || cfg->dist_type == SAQG_DIST_L2, "only L2 search is supported");
        const float m = cfg ? cfg->searcher_vars_bound_m : 4.0f;
        run_search(*index->impl, queries, nq, topk, nprobe, m, ids, dists, mem, (cudaStream_t)stream, stats, nullptr,
                   nprobe_per_query, topk_per_query);
    });
}

int saqg_search_static(const saqg_index *index, const float *queries, int64_t nq, int64_t topk, int64_t nprobe,
                       const saqg_searcher_config *cfg, uint32_t *ids, float *dists, void *stream) {
    return guarded([&] {
        SAQG_REQUIRE(index && queries && ids, "null argument");
        SAQG_REQUIRE(!cfg || cfg->dist_type == SAQG_DIST_L2, "only L2 search is supported");
        const float m = cfg ? cfg->searcher_vars_bound_m : 4.0f;
        run_search_static(*index->impl, queries, nq, topk, nprobe, m, ids, dists, (cudaStream_t)stream);
    });
}

int saqg_search_tc(const saqg_index *index, const float *queries, int64_t nq, int64_t topk, int64_t nprobe,
                   int64_t shortlist, const saqg_searcher_config *cfg, uint32_t *ids, float *dists, float *approx,
                   int mem, void *stream, saqg_tc_stats *stats) {
    return guarded([&] {
        SAQG_REQUIRE(index && (queries || nq == 0) && (ids || nq == 0), "null argument");
        SAQG_REQUIRE(!cfg || cfg->dist_type == SAQG_DIST_L2, "only L2 search is supported");
        SAQG_REQUIRE(mem == SAQG_MEM_HOST || mem == SAQG_MEM_DEVICE, "mem must be SAQG_MEM_HOST or SAQG_MEM_DEVICE");
        const float m = cfg ? cfg->searcher_vars_bound_m : 4.0f;
        run_search_tc(*index->impl, queries, nq, topk, nprobe, shortlist, m, ids, dists, approx, mem,
                      (cudaStream_t)stream, stats);
    });
}

int saqg_search_tc_batch(const saqg_index *index, const float *queries, int64_t nq, const int32_t *nprobe_per_query,
                         const int32_t *topk_per_query, int64_t nprobe, int64_t topk, int64_t shortlist,
                         const saqg_searcher_config *cfg, uint32_t *ids, float *dists, float *approx, int mem,
                         void *stream, saqg_tc_stats *stats) {
    return guarded([&] {
        SAQG_REQUIRE(index && (queries || nq == 0) && (ids || nq == 0), "null argument");
        SAQG_REQUIRE(!cfg || cfg->dist_type == SAQG_DIST_L2, "only L2 search is supported");
        SAQG_REQUIRE(mem == SAQG_MEM_HOST || mem == SAQG_MEM_DEVICE, "mem must be SAQG_MEM_HOST or SAQG_MEM_DEVICE");
        const float m = cfg ? cfg->searcher_vars_bound_m : 4.0f;
        run_search_tc(*index->impl, queries, nq, topk, nprobe, shortlist, m, ids, dists, approx, mem,
                      (cudaStream_t)stream, stats, nprobe_per_query, topk_per_query);
    });
}

int saqg_search_graph_create(const saqg_index *index, const float *queries, int64_t nq, int64_t topk, int64_t nprobe,
                             const saqg_searcher_config *cfg, uint32_t *ids, float *dists, void *stream,
                             saqg_search_graph **out) {
    return guarded([&] {
        SAQG_REQUIRE(index && queries && ids && out, "null argument");
        SAQG_REQUIRE(!cfg || cfg->dist_type == SAQG_DIST_L2, "only L2 search is supported");
        *out = nullptr;
        const float m = cfg ? cfg->searcher_vars_bound_m : 4.0f;
        SearchGraph *g = graph_create(*index->impl, nq, topk, nprobe, m, queries, ids, dists, (cudaStream_t)stream,
                                      GraphCfg{});
        *out = new saqg_search_graph{g};
    });
}

namespace {
void fill_report(saqg_tune_report *r, int form, const TuneReport &t) {
    if (!r) return;
    r->form = form;
    r->scan_mode = t.scan.mode;
    r->defer_blocks = t.scan.defer_blocks;
    r->first_blocks = t.scan.first_blocks;
    r->spec_levels = t.scan.spec_levels;
    r->pairs_per_chunk = t.tc.bn;
    r->candidates = t.candidates;
    r->default_ms = t.default_ms;
    r->tuned_ms = t.tuned_ms;
}
}  // namespace

int saqg_autotune(const saqg_index *index, const float *queries, int64_t nq, int64_t topk, int64_t nprobe,
                  int64_t shortlist, int form, const saqg_searcher_config *cfg, void *stream,
                  saqg_tune_report *report) {
    return guarded([&] {
        SAQG_REQUIRE(index && queries, "null argument");
        SAQG_REQUIRE(form == SAQG_FORM_EXACT || form == SAQG_FORM_TC, "unknown search form");
        SAQG_REQUIRE(!cfg || cfg->dist_type == SAQG_DIST_L2, "only L2 search is supported");
        const float m = cfg ? cfg->searcher_vars_bound_m : 4.0f;
        const TuneReport t =
            form == SAQG_FORM_EXACT
                ? autotune_exact(*index->impl, queries, nq, topk, nprobe, m, (cudaStream_t)stream)
                : autotune_tc(*index->impl, queries, nq, topk, nprobe, shortlist, m, (cudaStream_t)stream);
        fill_report(report, form, t);
    });
}

int saqg_search_graph_create_ex(const saqg_index *index, const float *queries, int64_t nq, int64_t topk,
                                int64_t nprobe, const saqg_searcher_config *cfg, const saqg_graph_config *gcfg,
                                uint32_t *ids, float *dists, void *stream, saqg_search_graph **out,
                                saqg_tune_report *report) {
    return guarded([&] {
        SAQG_REQUIRE(index && queries && ids && out && gcfg, "null argument");
        SAQG_REQUIRE(!cfg || cfg->dist_type == SAQG_DIST_L2, "only L2 search is supported");
        *out = nullptr;
        const float m = cfg ? cfg->searcher_vars_bound_m : 4.0f;
        GraphCfg gc;
        gc.form = gcfg->form;
        gc.np_dev = gcfg->nprobe_per_query;
        gc.k_dev = gcfg->topk_per_query;
        gc.shortlist = gcfg->shortlist;
        gc.cand_cap = gcfg->candidate_capacity;
        gc.autotune = gcfg->autotune;
        SearchGraph *g = graph_create(*index->impl, nq, topk, nprobe, m, queries, ids, dists, (cudaStream_t)stream, gc);
        fill_report(report, gc.form, graph_tune(g));
        *out = new saqg_search_graph{g};
    });
}

int saqg_search_graph_status(saqg_search_graph *graph, void *stream) {
    return guarded([&] {
        SAQG_REQUIRE(graph, "null argument");
        graph_status(graph->impl, (cudaStream_t)stream);
    });
}

int saqg_search_graph_launch(saqg_search_graph *graph, void *stream) {
    return guarded([&] {
        SAQG_REQUIRE(graph, "null argument");
        graph_launch(graph->impl, (cudaStream_t)stream);
    });
}

int saqg_search_graph_free(saqg_search_graph *graph) {
    return guarded([&] {
        if (!graph) return;
        graph_free(graph->impl);
        delete graph;
    });
}

int saqg_server_create(const saqg_index *index, const saqg_server_config *cfg, saqg_server **out) {
    return guarded([&] {
        SAQG_REQUIRE(index && out, "null argument");
        *out = nullptr;
        Server *s = server_create(*index->impl, cfg);
        *out = new saqg_server{s};
    });
}

int saqg_server_submit(saqg_server *server, const float *query, int32_t nprobe, int32_t topk, uint64_t *ticket) {
    return guarded([&] {
        SAQG_REQUIRE(server && query && ticket, "null argument");
        *ticket = server_submit(server->impl, query, nprobe, topk);
    });
}

int saqg_server_wait(saqg_server *server, uint64_t ticket, uint32_t *ids, float *dists, double *latency_ms,
                     int32_t timeout_ms) {
    return guarded([&] {
        SAQG_REQUIRE(server, "null argument");
        server_wait(server->impl, ticket, ids, dists, latency_ms, timeout_ms);
    });
}

int saqg_server_get_stats(saqg_server *server, saqg_server_stats *out) {
    return guarded([&] {
        SAQG_REQUIRE(server && out, "null argument");
        server_stats(server->impl, out);
    });
}

int saqg_server_run_trace(saqg_server *server, const float *queries, int64_t n, const double *arrival_s,
                          const int32_t *nprobe, const int32_t *topk, int32_t row, uint32_t *ids, float *dists,
                          double *latency_ms) {
    return guarded([&] {
        SAQG_REQUIRE(server && queries && arrival_s && nprobe && topk, "null argument");
        SAQG_REQUIRE(n >= 0 && row >= 1, "bad trace shape");
        server_run_trace(server->impl, queries, n, arrival_s, nprobe, topk, row, ids, dists, latency_ms);
    });
}

int saqg_server_free(saqg_server *server) {
    return guarded([&] {
        if (!server) return;
        server_free(server->impl);
        delete server;
    });
}

int saqg_estimate(const saqg_index *index, const float *query_host, int64_t nprobe, const saqg_searcher_config *cfg,
                  uint32_t *ids, float *acc, float *fast, float *vars, int64_t cap, int64_t *count) {
    return guarded([&] {
        SAQG_REQUIRE(index && query_host && count, "null argument");
        SAQG_REQUIRE(cap == 0 || (ids && acc && fast && vars), "null output buffer");
        SAQG_REQUIRE(!cfg || cfg->dist_type == SAQG_DIST_L2, "only L2 estimation is supported");
        const float m = cfg ? cfg->searcher_vars_bound_m : 4.0f;
        *count = run_estimate(*index->impl, query_host, nprobe, m, ids, acc, fast, vars, cap);
    });
}

int saqg_plan(const float *variance_host, int64_t dim_padded, float avg_bits, int enable_segmentation, int seg_eqseg,
              int64_t *dims, int64_t *bits, int cap, int *num_segments) {
    return guarded([&] {
        SAQG_REQUIRE(num_segments && (cap == 0 || (dims && bits)), "null argument");
        SAQG_REQUIRE(dim_padded > 0 && dim_padded % 64 == 0, "dim_padded must be a positive multiple of 64");
        SAQG_REQUIRE(avg_bits >= 0 && avg_bits <= kMaxBits, "avg_bits out of range");
        SAQG_REQUIRE(!enable_segmentation || seg_eqseg > 0 || variance_host, "variance required for the DP planner");
        auto p = make_plan(variance_host, dim_padded, avg_bits, enable_segmentation != 0, seg_eqseg);
        *num_segments = (int)p.size();
        for (int i = 0; i < (int)p.size() && i < cap; ++i) {
            dims[i] = p[i].first;
            bits[i] = p[i].second;
        }
    });
}

int saqg_plan_gpu(const float *variance, int64_t dim_padded, float avg_bits, int enable_segmentation, int seg_eqseg,
                  int mem, void *stream, int64_t *dims, int64_t *bits, int cap, int *num_segments) {
    return guarded([&] {
        SAQG_REQUIRE(num_segments && (cap == 0 || (dims && bits)), "null argument");
        SAQG_REQUIRE(dim_padded > 0 && dim_padded % 64 == 0, "dim_padded must be a positive multiple of 64");
        SAQG_REQUIRE(avg_bits >= 0 && avg_bits <= kMaxBits, "avg_bits out of range");
        SAQG_REQUIRE(mem == SAQG_MEM_HOST || mem == SAQG_MEM_DEVICE, "mem must be SAQG_MEM_HOST or SAQG_MEM_DEVICE");
        SAQG_REQUIRE(!enable_segmentation || seg_eqseg > 0 || variance, "variance required for the DP planner");
        auto p = make_plan_gpu(variance, dim_padded, avg_bits, enable_segmentation != 0, seg_eqseg,
                               mem == SAQG_MEM_DEVICE, (cudaStream_t)stream);
        *num_segments = (int)p.size();
        for (int i = 0; i < (int)p.size() && i < cap; ++i) {
            dims[i] = p[i].first;
            bits[i] = p[i].second;
        }
    });
}

int saqg_caq_encode(const float *resid, int64_t n, int64_t dim, int bits, const float *centroid, int rd_lmt, float eps,
                    int32_t *codes, float *factors, int mem, void *stream) {
    return guarded([&] {
        SAQG_REQUIRE(resid && codes && factors, "null argument");
        SAQG_REQUIRE(n >= 0 && dim > 1 && dim % 64 == 0, "dim must be a multiple of 64");
        SAQG_REQUIRE(bits >= 0 && bits <= kMaxBits, "bits must be in [0, 13]");
        SAQG_REQUIRE(mem == SAQG_MEM_HOST || mem == SAQG_MEM_DEVICE, "bad mem flag");
        run_caq_encode(resid, n, dim, bits, centroid, rd_lmt, eps, codes, factors, mem, (cudaStream_t)stream);
    });
}

}  // extern "C"
