/* GpuIVF: the reference's saqlib::IVF member calls (saqlib/index/ivf.hpp:27-121)
 * over the C ABI of saqg.h, for C++ applications that switch a driver such as
 * src/test_qps.cpp or unit_test/ut_ivf_recall.cpp to the GPU by replacing the
 * IVF member.  Header-only; include with -I <repo>/include and link with
 * -L <repo>/saq_gb300/_lib -lsaqg.
 *
 * `RowVec` stands for the reference's Eigen::RowVectorXf and `Cfg` for its
 * SearcherConfig: only .data() and .searcher_vars_bound_m are used, so no
 * Eigen header is needed here.  Where the reference aborts through glog CHECK,
 * these members throw std::runtime_error with saqg_last_error()'s text. */
#ifndef SAQG_IVF_HPP
#define SAQG_IVF_HPP

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "saqg.h"

class GpuIVF {
    saqg_index *h_ = nullptr;

    static void check(int status) {
        if (status != SAQG_OK) throw std::runtime_error(saqg_last_error());
    }

  public:
    /* IVF::load (ivf.hpp:230-264): a file written by the reference's IVF::save
     * or by saqg_index_save / saqg_index_save_v2. */
    explicit GpuIVF(const char *index_path) { check(saqg_index_load(index_path, &h_)); }
    GpuIVF(const GpuIVF &) = delete;
    GpuIVF &operator=(const GpuIVF &) = delete;
    ~GpuIVF() { saqg_index_free(h_); }

    /* IVF::save (ivf.hpp:197-228), the reference's format byte for byte. */
    void save(const char *path) const { check(saqg_index_save(h_, path)); }

    /* IVF::search<L2Sqr> (ivf.hpp:91-94, 275-311): the same argument meaning;
     * `results` receives topk ids, 0 where the pool was not filled.  Host
     * memory, the caller's thread; answers are the reference's bit for bit. */
    template <class RowVec, class Cfg>
    void search(const RowVec &q, size_t topk, size_t nprobe, const Cfg &cfg, uint32_t *results) const {
        saqg_searcher_config c{cfg.searcher_vars_bound_m, SAQG_DIST_L2};
        check(saqg_search(h_, q.data(), 1, (int64_t)topk, (int64_t)nprobe, &c, results, nullptr, SAQG_MEM_HOST,
                          nullptr));
    }

    /* A batch of nq row-major queries in one call (each row answered as its own
     * IVF::search call); `results` is nq x topk, `dists` (optional) the same. */
    template <class Cfg>
    void search_batch(const float *queries, size_t nq, size_t topk, size_t nprobe, const Cfg &cfg,
                      uint32_t *results, float *dists = nullptr) const {
        saqg_searcher_config c{cfg.searcher_vars_bound_m, SAQG_DIST_L2};
        check(saqg_search(h_, queries, (int64_t)nq, (int64_t)topk, (int64_t)nprobe, &c, results, dists,
                          SAQG_MEM_HOST, nullptr));
    }

    saqg_index *handle() const { return h_; }
};

#endif /* SAQG_IVF_HPP */
