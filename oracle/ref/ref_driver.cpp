// Test-infrastructure driver around the UNMODIFIED reference headers (saqlib/).
//
// It is compiled in the development container only (the reference is x86 +
// AVX-512 code and is not present on the GPU machines) and produces the golden
// vectors under tests/golden/ and the reference CPU timings. Nothing in the
// product links or runs it.
//
// Sub-commands (all arrays are raw little-endian binaries):
//   build    data.f32 N D centroids.f32 K cids.u32 out.index avg_bits seg eqseg rotate rdlmt eps threads [vars.f32]
//   search   index queries.f32 NQ topk nprobe vars_m out_ids.u32 out_ms.f32 threads
//   estimate index queries.f32 NQ nprobe vars_m out_prefix
//   dump     index queries.f32 NQ nprobe out_prefix
//   encode   resid.f32 n D bits centroid.f32 rdlmt out_prefix
//   plan     vars.f32 D avg_bits seg eqseg out.txt
//
// The reference's private members are opened with the usual test-only
// `#define private public` so that internal LUTs and sums can be dumped
// without changing a line of the reference.
#include <bits/stdc++.h>
#include <immintrin.h>
#include <thread>

#include "third/Eigen/Dense"

#define private public
#define protected public
#include "index/ivf.hpp"
#undef private
#undef protected

using namespace saqlib;

template <class T>
static std::vector<T> read_raw(const char *path, size_t count) {
    std::vector<T> v(count);
    FILE *f = std::fopen(path, "rb");
    if (!f) { std::fprintf(stderr, "cannot open %s\n", path); std::exit(2); }
    size_t got = std::fread(v.data(), sizeof(T), count, f);
    std::fclose(f);
    if (got != count) { std::fprintf(stderr, "short read %s: %zu of %zu\n", path, got, count); std::exit(2); }
    return v;
}

template <class T>
static void write_raw(const std::string &path, const T *p, size_t count) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) { std::fprintf(stderr, "cannot write %s\n", path.c_str()); std::exit(2); }
    std::fwrite(p, sizeof(T), count, f);
    std::fclose(f);
}

// ---------------------------------------------------------------------------
// Harness-side cluster quantizer. For segments with >1 bit it is exactly
// QuantizerCluster::quantize. For 1-bit segments the reference never fills
// QuantBaseCode::code (caq_encoder.hpp:239-246) and the packer then reads an
// empty vector; here the code from CAQEncoder::encode is handed to the packer
// as the top (and only) bit, which is what the layout expects.
// ---------------------------------------------------------------------------
static void harness_quantize_segment(const QuantizerCluster &qc, const FloatRowMat &or_vecs, const FloatVec &centroid,
                                     CAQClusterData &clus) {
    if (qc.num_bits_ != 1) {
        qc.quantize(or_vecs, centroid, clus);
        return;
    }
    const auto *data = qc.data_;
    FloatRowMat o_vecs;
    if (data->rotator) {
        clus.centroid() = centroid * data->rotator->get_P();
        o_vecs = (or_vecs * data->rotator->get_P()).rowwise() - clus.centroid();
    } else {
        clus.centroid() = centroid;
        o_vecs = or_vecs.rowwise() - clus.centroid();
    }
    CAQEncoder encoder(qc.num_dim_pad_, qc.num_bits_, data->cfg);
    ClusterPacker packer(qc.num_dim_pad_, qc.num_bits_, clus, data->cfg.use_fastscan);
    QuantBaseCode base_code;
    for (size_t i = 0; i < clus.num_vec(); ++i) {
        FloatVec curr_vec = o_vecs.row(i);
        encoder.encode_and_fac(curr_vec, base_code, &centroid);
        CaqCode caq;
        encoder.encode(curr_vec, caq);
        base_code.code = caq.code;
        packer.store_and_pack(i, base_code);
    }
    packer.finalize_and_store();
}

static void harness_construct(IVF &ivf, const FloatRowMat &data, const FloatRowMat &centroids, const PID *cids,
                              int threads) {
    bool has_one_bit = false;
    {
        // The plan is known only after the variance is set; replicate construct() steps 1-2.
        ivf.prepare_initer(&centroids);
        if (!ivf.saq_data_maker_->is_variance_set()) ivf.saq_data_maker_->compute_variance(data);
        ivf.saq_data_ = ivf.saq_data_maker_->return_data();
        for (auto &[d, b] : ivf.saq_data_->quant_plan) has_one_bit |= (b == 1);
    }
    std::vector<std::vector<PID>> id_lists(ivf.num_cen_);
    std::vector<size_t> counts(ivf.num_cen_, 0);
    for (size_t i = 0; i < ivf.num_data_; ++i) {
        id_lists[cids[i]].push_back((PID)i);
        counts[cids[i]] += 1;
    }
    ivf.allocate_clusters(counts);
    SAQuantizer saq(ivf.saq_data_.get());
    BS::thread_pool pool(threads);
    for (size_t c = 0; c < ivf.num_cen_; ++c) {
        pool.detach_task([&, c]() {
            const FloatVec cur_centroid = centroids.row(c);
            auto &clu = ivf.parallel_clusters_[c];
            if (!has_one_bit) {
                saq.quantize_cluster(data, cur_centroid, id_lists[c], clu);
                return;
            }
            // SAQuantizer::quantize_cluster with the 1-bit segment fix above.
            std::copy(id_lists[c].begin(), id_lists[c].end(), clu.ids());
            const size_t num_points = clu.num_vec_;
            for (size_t ci = 0, offset = 0; ci < clu.num_segments_; ++ci) {
                auto &seg = clu.get_segment(ci);
                const size_t copy_size = std::min(seg.num_dim_padded_, saq.num_dim_ - offset);
                FloatRowMat vecs(num_points, seg.num_dim_padded_);
                vecs.setZero();
                for (size_t r = 0; r < num_points; ++r)
                    vecs.row(r).head(copy_size) = data.row(seg.ids()[r]).segment(offset, copy_size);
                FloatVec cen(seg.num_dim_padded_);
                cen.setZero();
                cen.head(copy_size) = cur_centroid.segment(offset, copy_size);
                harness_quantize_segment(*saq.data_quans_[ci], vecs, cen, seg);
                offset += seg.num_dim_padded_;
            }
        });
    }
    pool.wait();
}

static int cmd_build(int argc, char **argv) {
    if (argc < 16) return 1;
    size_t N = std::stoul(argv[3]), D = std::stoul(argv[4]), K = std::stoul(argv[6]);
    auto data_v = read_raw<float>(argv[2], N * D);
    auto cen_v = read_raw<float>(argv[5], K * D);
    auto cids = read_raw<PID>(argv[7], N);
    QuantizeConfig cfg;
    cfg.avg_bits = std::stof(argv[9]);
    cfg.enable_segmentation = std::stoi(argv[10]) != 0;
    cfg.seg_eqseg = std::stoi(argv[11]);
    cfg.single.random_rotation = std::stoi(argv[12]) != 0;
    cfg.single.caq_adj_rd_lmt = std::stoi(argv[13]);
    cfg.single.caq_adj_eps = std::stof(argv[14]);
    int threads = std::stoi(argv[15]);
    FloatRowMat data = Eigen::Map<FloatRowMat>(data_v.data(), N, D);
    FloatRowMat cen = Eigen::Map<FloatRowMat>(cen_v.data(), K, D);
    IVF ivf(N, D, K, cfg);
    if (argc > 16) {
        auto vars = read_raw<float>(argv[16], D);
        FloatVec v = Eigen::Map<FloatVec>(vars.data(), 1, D);
        ivf.set_variance(v);
    }
    auto t0 = std::chrono::steady_clock::now();
    harness_construct(ivf, data, cen, cids.data(), threads);
    double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    ivf.save(argv[8]);
    std::printf("{\"construct_s\": %.6f, \"plan\": [", sec);
    bool first = true;
    for (auto &[d, b] : ivf.saq_data_->quant_plan) {
        std::printf("%s[%zu, %zu]", first ? "" : ", ", d, b);
        first = false;
    }
    std::printf("], \"sizeof_QuantizeConfig\": %zu, \"sizeof_QuantSingleConfig\": %zu}\n", sizeof(QuantizeConfig),
                sizeof(QuantSingleConfig));
    return 0;
}

static int cmd_search(int argc, char **argv) {
    if (argc < 11) return 1;
    IVF ivf;
    ivf.load(argv[2]);
    size_t NQ = std::stoul(argv[4]), topk = std::stoul(argv[5]), nprobe = std::stoul(argv[6]);
    float m = std::stof(argv[7]);
    int threads = std::stoi(argv[10]);
    size_t D = ivf.num_dim_;
    auto q = read_raw<float>(argv[3], NQ * D);
    std::vector<PID> out(NQ * topk);
    std::vector<float> ms(NQ);
    SearcherConfig scfg;
    scfg.searcher_vars_bound_m = m;
    std::atomic<size_t> next{0};
    auto t0 = std::chrono::steady_clock::now();
    auto worker = [&]() {
        for (size_t i; (i = next.fetch_add(1)) < NQ;) {
            Eigen::RowVectorXf qv = Eigen::Map<Eigen::RowVectorXf>(q.data() + i * D, D);
            auto s = std::chrono::steady_clock::now();
            ivf.search<DistType::L2Sqr>(qv, topk, nprobe, scfg, out.data() + i * topk);
            ms[i] = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - s).count();
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t) th.emplace_back(worker);
    for (auto &t : th) t.join();
    double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    write_raw(argv[8], out.data(), out.size());
    write_raw(argv[9], ms.data(), ms.size());
    std::printf("{\"wall_s\": %.6f, \"qps_wall\": %.3f, \"threads\": %d}\n", wall, NQ / wall, threads);
    return 0;
}

static int cmd_estimate(int argc, char **argv) {
    if (argc < 8) return 1;
    IVF ivf;
    ivf.load(argv[2]);
    size_t NQ = std::stoul(argv[4]), nprobe = std::stoul(argv[5]);
    float m = std::stof(argv[6]);
    std::string pre = argv[7];
    size_t D = ivf.num_dim_;
    auto q = read_raw<float>(argv[3], NQ * D);
    SearcherConfig scfg;
    scfg.searcher_vars_bound_m = m;
    std::vector<PID> ids;
    std::vector<float> acc, fast, vars;
    std::vector<uint64_t> counts;
    for (size_t i = 0; i < NQ; ++i) {
        Eigen::RowVectorXf qv = Eigen::Map<Eigen::RowVectorXf>(q.data() + i * D, D);
        std::vector<std::pair<PID, float>> dl;
        std::vector<float> fl, vl;
        ivf.estimate<DistType::L2Sqr>(qv, nprobe, scfg, dl, &fl, &vl);
        counts.push_back(dl.size());
        for (auto &[id, d] : dl) { ids.push_back(id); acc.push_back(d); }
        fast.insert(fast.end(), fl.begin(), fl.end());
        vars.insert(vars.end(), vl.begin(), vl.end());
    }
    write_raw(pre + ".count.u64", counts.data(), counts.size());
    write_raw(pre + ".ids.u32", ids.data(), ids.size());
    write_raw(pre + ".acc.f32", acc.data(), acc.size());
    write_raw(pre + ".fast.f32", fast.data(), fast.size());
    write_raw(pre + ".vars.f32", vars.data(), vars.size());
    return 0;
}

// Per query: probe order and centroid distances; per segment the rotated query
// and prune bound; per (probe, segment) the LUT scalars, u16 LUT and the
// integer FastScan sums of every block.
static int cmd_dump(int argc, char **argv) {
    if (argc < 7) return 1;
    IVF ivf;
    ivf.load(argv[2]);
    size_t NQ = std::stoul(argv[4]), nprobe = std::stoul(argv[5]);
    std::string pre = argv[6];
    size_t D = ivf.num_dim_;
    auto q = read_raw<float>(argv[3], NQ * D);
    std::vector<PID> probe_ids;
    std::vector<float> probe_d, rotq, prune, scal;
    std::vector<uint16_t> luts;
    std::vector<int32_t> sums;
    SearcherConfig scfg;
    for (size_t i = 0; i < NQ; ++i) {
        Eigen::RowVectorXf qv = Eigen::Map<Eigen::RowVectorXf>(q.data() + i * D, D);
        std::vector<Candidate> cd(nprobe);
        ivf.initer_->centroids_distances(qv, nprobe, DistType::L2Sqr, cd);
        for (auto &c : cd) { probe_ids.push_back(c.id); probe_d.push_back(c.distance); }
        SaqCluEstimator<DistType::L2Sqr> est(*ivf.saq_data_, scfg, qv);
        for (auto &e : est.estimators_) {
            rotq.insert(rotq.end(), e.query_data_.data(), e.query_data_.data() + e.query_data_.size());
            prune.push_back(e.without_ip_prune_bound_);
        }
        for (size_t p = 0; p < nprobe; ++p) {
            auto &clu = ivf.parallel_clusters_[cd[p].id];
            est.prepare(&clu);
            for (size_t s = 0; s < est.estimators_.size(); ++s) {
                auto &e = est.estimators_[s];
                auto &lut = e.lut_;
                scal.push_back(lut.delta_);
                scal.push_back(lut.sum_vl_lut_);
                scal.push_back(lut.sum_q_);
                scal.push_back(lut.q_l2sqr_);
                scal.push_back(lut.q_l2norm_);
                if (e.num_bits_ == 0) continue;
                // Undo transfer_lut_hacc: group of 4 codebooks = 64 lo bytes then 64 hi bytes.
                size_t ncb = e.num_dim_padded_ / 4;
                for (size_t cb = 0; cb < ncb; ++cb) {
                    const uint8_t *lo = lut.lut_.data() + (cb / 4) * 128 + (cb % 4) * 16;
                    for (int j = 0; j < 16; ++j) luts.push_back(uint16_t(lo[j] | (lo[j + 64] << 8)));
                }
                auto &seg = clu.get_segment(s);
                for (size_t b = 0; b < seg.num_blocks(); ++b) {
                    __m512i res[2];
                    fastscan::accumulate_hacc(seg.short_code(b), lut.lut_.data(), res, e.num_dim_padded_);
                    int32_t tmp[32];
                    _mm512_storeu_si512(tmp, res[0]);
                    _mm512_storeu_si512(tmp + 16, res[1]);
                    sums.insert(sums.end(), tmp, tmp + 32);
                }
            }
        }
    }
    write_raw(pre + ".probe_ids.u32", probe_ids.data(), probe_ids.size());
    write_raw(pre + ".probe_d.f32", probe_d.data(), probe_d.size());
    write_raw(pre + ".rotq.f32", rotq.data(), rotq.size());
    write_raw(pre + ".prune.f32", prune.data(), prune.size());
    write_raw(pre + ".scal.f32", scal.data(), scal.size());
    write_raw(pre + ".lut.u16", luts.data(), luts.size());
    write_raw(pre + ".sums.i32", sums.data(), sums.size());
    return 0;
}

// CAQ encode + pack of given residual vectors (one cluster, one segment).
static int cmd_encode(int argc, char **argv) {
    if (argc < 9) return 1;
    size_t n = std::stoul(argv[3]), D = std::stoul(argv[4]), bits = std::stoul(argv[5]);
    auto r = read_raw<float>(argv[2], n * D);
    auto c = read_raw<float>(argv[6], D);
    QuantSingleConfig cfg;
    cfg.caq_adj_rd_lmt = std::stoi(argv[7]);
    std::string pre = argv[8];
    FloatVec cen = Eigen::Map<FloatVec>(c.data(), 1, D);
    std::vector<std::pair<size_t, size_t>> plan{{D, bits}};
    SaqCluData saq(n, plan, false);
    auto &clus = saq.get_segment(0);
    CAQEncoder encoder(D, bits, cfg);
    ClusterPacker packer(D, bits, clus, true);
    std::vector<int32_t> codes;
    std::vector<double> facs; // o_l2norm, ip_cent_oa, rescale, error (as stored, widened)
    QuantBaseCode base_code;
    for (size_t i = 0; i < n; ++i) {
        FloatVec v = Eigen::Map<FloatVec>(r.data() + i * D, 1, D);
        encoder.encode_and_fac(v, base_code, &cen);
        CaqCode caq;
        encoder.encode(v, caq);
        if (bits == 1) base_code.code = caq.code;
        for (size_t j = 0; j < D; ++j) codes.push_back(bits ? caq.code[j] : 0);
        facs.push_back(base_code.o_l2norm);
        facs.push_back(base_code.ip_cent_oa);
        facs.push_back(base_code.fac_rescale);
        facs.push_back(base_code.fac_error);
        packer.store_and_pack(i, base_code);
    }
    packer.finalize_and_store();
    write_raw(pre + ".codes.i32", codes.data(), codes.size());
    write_raw(pre + ".facs.f64", facs.data(), facs.size());
    // block area (factors + packed short codes) and per-vector long codes, as laid out in memory
    size_t blk_bytes = saq.shortb_code_bytes_;
    write_raw(pre + ".blocks.u8", saq.short_code_, blk_bytes * saq.num_blocks_);
    write_raw(pre + ".long.u8", saq.long_code_, saq.longb_code_bytes_ * n);
    write_raw(pre + ".exfac.f32", reinterpret_cast<float *>(saq.long_factors_), 2 * n);
    return 0;
}

static int cmd_plan(int argc, char **argv) {
    if (argc < 8) return 1;
    size_t D = std::stoul(argv[3]);
    auto vars = read_raw<float>(argv[2], D);
    QuantizeConfig cfg;
    cfg.avg_bits = std::stof(argv[4]);
    cfg.enable_segmentation = std::stoi(argv[5]) != 0;
    cfg.seg_eqseg = std::stoi(argv[6]);
    cfg.single.random_rotation = false;
    SaqDataMaker maker(cfg, D);
    FloatVec v = Eigen::Map<FloatVec>(vars.data(), 1, D);
    maker.set_variance(v);
    FILE *f = std::fopen(argv[7], "w");
    for (auto &[d, b] : maker.get_data()->quant_plan) std::fprintf(f, "%zu %zu\n", d, b);
    std::fclose(f);
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 2) return 1;
    std::string c = argv[1];
    int rc = 1;
    if (c == "build") rc = cmd_build(argc, argv);
    else if (c == "search") rc = cmd_search(argc, argv);
    else if (c == "estimate") rc = cmd_estimate(argc, argv);
    else if (c == "dump") rc = cmd_dump(argc, argv);
    else if (c == "encode") rc = cmd_encode(argc, argv);
    else if (c == "plan") rc = cmd_plan(argc, argv);
    if (rc == 1) std::fprintf(stderr, "bad arguments for %s\n", c.c_str());
    return rc;
}
