// Index file I/O and upload: the reference's binary `.index` format
// (IVF::save/load, index/ivf.hpp:197-264) <-> the device layout of saqg_internal.h.
//
// The file layout (little-endian, size_t = 8 bytes) is the reference's, kept
// byte for byte so that files move freely between the two implementations:
//   [N][D][K] | centroids K x D f32 | QuantizeConfig (32 raw bytes) | num_dim |
//   variance (size_t n, n x f32) | #segments | per segment: dim_pad, bits,
//   QuantSingleConfig (20 raw bytes), rotator flag (1 byte), P (dim x dim f32) |
//   cluster sizes K x size_t | per cluster: short factors (multi-segment only),
//   short code blocks, long codes, long factors, ids, rotated centroids.
// IVF::load reads every cluster K times in a nested loop (ivf.hpp:256-260,
// harmless only because reads past EOF are no-ops); here each is read once.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <memory>

#include "saqg_internal.h"

namespace saqg {

namespace {
const int kPerm0[16] = {0, 8, 1, 9, 2, 10, 3, 11, 4, 12, 5, 13, 6, 14, 7, 15};

struct Reader {
    FILE *f;
    std::string path;
    void read(void *p, size_t n) {
        if (n && std::fread(p, 1, n, f) != n)
            throw Error{SAQG_ERR_IO, "truncated index file " + path};
    }
    uint64_t u64() {
        uint64_t v;
        read(&v, 8);
        return v;
    }
};

// Bytes of one segment's pieces (cluster_data.hpp:71-80, 206-294).
struct SegSizes {
    std::vector<int64_t> sc, pv, loff, scoff;
    int64_t block_bytes = 0, long_stride = 0;
};

SegSizes seg_sizes(const std::vector<Index::SegHost> &segs, bool compact) {
    SegSizes z;
    const size_t S = segs.size();
    z.sc.resize(S);
    z.pv.resize(S);
    z.loff.resize(S);
    z.scoff.resize(S);
    for (size_t s = 0; s < S; ++s) {
        z.sc[s] = segs[s].bits ? segs[s].dim * kBlock / 8 : 0;
        z.pv[s] = segs[s].bits ? segs[s].dim * (segs[s].bits - 1) / 8 : 0;
    }
    if (S == 1) {
        z.block_bytes = 64 * 4 + z.sc[0];
        z.long_stride = z.pv[0];
    } else {
        for (size_t s = 0; s < S; ++s) {
            z.scoff[s] = z.block_bytes;
            z.block_bytes += z.sc[s];
            z.loff[s] = z.long_stride;
            z.long_stride += compact ? z.pv[s] : (z.pv[s] + 15) / 16 * 16;
        }
    }
    return z;
}

int64_t lstride_of(int64_t pv) { return (pv + 15) / 16 * 16; }

// An index in host memory, arrays already in the device layout of
// saqg_internal.h (what load uploads and save downloads).
struct HostIndex {
    int64_t N = 0, D = 0, K = 0;
    uint8_t qcfg_raw[32] = {0};
    std::vector<float> var;
    std::vector<Index::SegHost> segs;
    bool compact = false;
    std::vector<int64_t> sizes;
    std::vector<float> cent;
    std::vector<uint32_t> ids;
    std::vector<std::vector<uint8_t>> codes, lcode;
    std::vector<std::vector<float>> onorm, ipc, rcent, exfac;
};
}  // namespace

Index::~Index() {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(device);
    ctx_pool.clear();  // on this index's device
    for (void *p : allocations) cudaFree(p);
    if (cnorm2) cudaFree(cnorm2);
    if (cent_bf16) cudaFree(cent_bf16);
    if (tc_codes) cudaFree(tc_codes);
    if (tc_tiles) cudaFree(tc_tiles);
    cudaSetDevice(cur);
}

CtxLease::CtxLease(const Index &I, cudaStream_t stream) : st(stream) {
    {
        std::lock_guard<std::mutex> lk(I.pool_mu);
        for (int pass = 0; pass < 2 && !c; ++pass)  // an idle context last used on this stream, else any idle one
            for (auto &p : I.ctx_pool)
                if ((pass == 1 || p->last_stream == stream) && p->mu.try_lock()) {
                    c = p.get();
                    break;
                }
        if (!c) {
            I.ctx_pool.push_back(std::make_unique<SearchCtx>());
            c = I.ctx_pool.back().get();
            c->mu.lock();
        }
    }
    try {
        if (!c->ev_done) SAQG_CUDA_TRY(cudaEventCreateWithFlags(&c->ev_done, cudaEventDisableTiming));
        if (c->used && c->last_stream != stream) SAQG_CUDA_TRY(cudaStreamWaitEvent(stream, c->ev_done, 0));
    } catch (...) {
        c->mu.unlock();
        throw;
    }
}

CtxLease::~CtxLease() {
    if (cudaEventRecord(c->ev_done, st) == cudaSuccess) {
        c->last_stream = st;
        c->used = true;
    } else {  // the next call cannot order itself after this one: let it wait for the device
        cudaGetLastError();
        cudaDeviceSynchronize();
        c->used = false;
    }
    c->mu.unlock();
}

SearchCtx::~SearchCtx() {
    if (ev_done) cudaEventDestroy(ev_done);
    if (scratch) cudaFree(scratch);
    if (split_scratch) cudaFree(split_scratch);
    if (aux) cudaStreamDestroy(aux);
    if (low) cudaStreamDestroy(low);
    if (ev_qfork) cudaEventDestroy(ev_qfork);
    if (ev_qjoin) cudaEventDestroy(ev_qjoin);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
}

void *Index::dalloc(size_t bytes) {
    void *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) throw Error{SAQG_ERR_NOMEM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e)};
    allocations.push_back(p);
    device_bytes += (int64_t)bytes;
    return p;
}

void Index::upload(void *dst, const void *src, size_t bytes) {
    if (bytes) SAQG_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
}

static void *grow(void *&buf, size_t &have, size_t bytes) {
    if (bytes > have) {
        // previous work on this buffer may still be in flight on any stream
        SAQG_CUDA_TRY(cudaDeviceSynchronize());
        if (buf) SAQG_CUDA_TRY(cudaFree(buf));
        buf = nullptr;
        have = 0;
        const size_t want = bytes + bytes / 4 + (1 << 20);
        cudaError_t e = cudaMalloc(&buf, want);
        if (e != cudaSuccess) throw Error{SAQG_ERR_NOMEM, std::string("scratch cudaMalloc failed: ") + cudaGetErrorString(e)};
        have = want;
    }
    return buf;
}

void *SearchCtx::scratch_get(size_t bytes) { return grow(scratch, scratch_bytes, bytes); }
void *SearchCtx::split_scratch_get(size_t bytes) { return grow(split_scratch, split_scratch_bytes, bytes); }

// The split pass is a batch's critical path: its stream gets the device's
// highest priority, so its CTAs go first while the CTA scan beside it fills in.
cudaStream_t SearchCtx::aux_stream() {
    if (!aux) {
        int least = 0, greatest = 0;
        SAQG_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        SAQG_CUDA_TRY(cudaStreamCreateWithPriority(&aux, cudaStreamNonBlocking, greatest));
    }
    return aux;
}
// The query preparation runs beside the centroid ranking and is needed only by
// the scan: it takes the device's least priority (also the default one), and
// the ranking's shortlist and select, beside it, the greatest (aux_stream).
cudaStream_t SearchCtx::low_stream() {
    if (!low) {
        int least = 0, greatest = 0;
        SAQG_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        SAQG_CUDA_TRY(cudaStreamCreateWithPriority(&low, cudaStreamNonBlocking, least));
    }
    return low;
}
cudaEvent_t SearchCtx::qfork_event() {
    if (!ev_qfork) SAQG_CUDA_TRY(cudaEventCreateWithFlags(&ev_qfork, cudaEventDisableTiming));
    return ev_qfork;
}
cudaEvent_t SearchCtx::qjoin_event() {
    if (!ev_qjoin) SAQG_CUDA_TRY(cudaEventCreateWithFlags(&ev_qjoin, cudaEventDisableTiming));
    return ev_qjoin;
}
cudaEvent_t SearchCtx::fork_event() {
    if (!ev_fork) SAQG_CUDA_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    return ev_fork;
}
cudaEvent_t SearchCtx::join_event() {
    if (!ev_join) SAQG_CUDA_TRY(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    return ev_join;
}

int64_t Index::max_blocks_of_probes(int64_t nprobe) const {
    if (top_blocks_prefix.empty()) return 1;
    return std::max<int64_t>(1, top_blocks_prefix[std::min<int64_t>(nprobe, (int64_t)top_blocks_prefix.size() - 1)]);
}

void finalize_view(Index &idx) {
    {
        std::vector<int64_t> nb(idx.K);
        for (int64_t c = 0; c < idx.K; ++c) nb[c] = idx.blk_off[c + 1] - idx.blk_off[c];
        std::sort(nb.begin(), nb.end(), std::greater<int64_t>());
        idx.top_blocks_prefix.assign(idx.K + 1, 0);
        for (int64_t c = 0; c < idx.K; ++c) idx.top_blocks_prefix[c + 1] = idx.top_blocks_prefix[c] + nb[c];
    }
    DevIndexView &v = idx.view;
    v.S = (int)idx.segs.size();
    v.K = (int)idx.K;
    v.D = (int)idx.D;
    int off = 0;
    for (int s = 0; s < v.S; ++s) {
        v.seg[s].qoff = off;
        off += v.seg[s].dim;
        // Lut::compFastIP's constant (lut.hpp:89-119): float (4 / 0.8) times the
        // float of the double reciprocal of the float square root, each rounded
        // to nearest as IEEE hosts and the device do
        const float four_over = 4.0f / 0.8f;
        const float inv_sqrt = (float)(1.0 / (double)std::sqrt((float)v.seg[s].dim));
        v.seg[s].c2 = four_over * inv_sqrt;
    }
    v.Dtot = off;
}

HostIndex parse_reference(const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) throw Error{SAQG_ERR_IO, "cannot open index file " + path};
    std::unique_ptr<FILE, int (*)(FILE *)> guard(f, std::fclose);
    Reader r{f, path};
    auto idx = std::make_unique<HostIndex>();
    idx->N = (int64_t)r.u64();
    idx->D = (int64_t)r.u64();
    idx->K = (int64_t)r.u64();
    if (idx->D <= 0 || idx->K <= 0 || idx->N < 0 || idx->D > (1 << 20) || idx->K > (1 << 28))
        throw Error{SAQG_ERR_IO, "implausible header in " + path};
    std::vector<float> &cent = idx->cent;
    cent.resize(idx->K * idx->D);
    r.read(cent.data(), 4 * cent.size());
    r.read(idx->qcfg_raw, 32);
    int64_t num_dim = (int64_t)r.u64();
    int64_t nv = (int64_t)r.u64();
    if (num_dim != idx->D || nv != num_dim)
        throw Error{SAQG_ERR_IO, "variance / dimension mismatch in " + path};
    idx->var.resize(nv);
    r.read(idx->var.data(), 4 * nv);
    int64_t nseg = (int64_t)r.u64();
    if (nseg < 1 || nseg > kMaxSeg) throw Error{SAQG_ERR_IO, "unsupported segment count in " + path};
    int64_t dsum = 0;
    for (int64_t s = 0; s < nseg; ++s) {
        Index::SegHost sg;
        sg.dim = (int64_t)r.u64();
        sg.bits = (int64_t)r.u64();
        r.read(sg.cfg_raw, 20);
        uint8_t flag = 0;
        r.read(&flag, 1);
        if (sg.dim <= 0 || sg.dim % 64 || sg.bits > kMaxBits || sg.dim > 16384)
            throw Error{SAQG_ERR_IO, "unsupported segment in " + path};
        sg.rotated = flag != 0;
        if (sg.rotated) {
            sg.P.resize(sg.dim * sg.dim);
            r.read(sg.P.data(), 4 * sg.P.size());
        }
        dsum += sg.dim;
        idx->segs.push_back(std::move(sg));
    }
    if (dsum < idx->D || idx->D % 64 != 0)
        throw Error{SAQG_ERR_IO, "dimension must be a multiple of 64 (the reference's load requires it)"};
    idx->compact = nseg == 1 || idx->qcfg_raw[9] != 0;
    idx->sizes.resize(idx->K);
    r.read(idx->sizes.data(), 8 * idx->K);
    std::vector<int64_t> blk_off(idx->K + 1, 0), vec_off(idx->K + 1, 0);
    for (int64_t c = 0; c < idx->K; ++c) {
        if (idx->sizes[c] < 0) throw Error{SAQG_ERR_IO, "negative cluster size in " + path};
        blk_off[c + 1] = blk_off[c] + (idx->sizes[c] + kBlock - 1) / kBlock;
        vec_off[c + 1] = vec_off[c] + idx->sizes[c];
    }
    if (vec_off[idx->K] != idx->N) throw Error{SAQG_ERR_IO, "cluster sizes do not sum to N in " + path};
    const int64_t NB = blk_off[idx->K], N = idx->N;
    const SegSizes z = seg_sizes(idx->segs, idx->compact);
    const size_t S = idx->segs.size();

    // host staging of the device layout
    auto &codes = idx->codes, &lcode = idx->lcode;
    auto &onorm = idx->onorm, &ipc = idx->ipc, &rcent = idx->rcent, &exfac = idx->exfac;
    codes.resize(S);
    lcode.resize(S);
    onorm.resize(S);
    ipc.resize(S);
    rcent.resize(S);
    exfac.resize(S);
    for (size_t s = 0; s < S; ++s) {
        const int64_t dim = idx->segs[s].dim;
        codes[s].assign(idx->segs[s].bits ? NB * kBlock * dim / 8 : 0, 0);
        onorm[s].assign(NB * kBlock, 0.0f);
        ipc[s].assign(NB * kBlock, 0.0f);
        lcode[s].assign(N * lstride_of(z.pv[s]), 0);
        exfac[s].assign(2 * N, 0.0f);
        rcent[s].assign(idx->K * dim, 0.0f);
    }
    std::vector<uint32_t> &ids = idx->ids;
    ids.resize(N);
    std::vector<float> sfac, blk, lfac;
    std::vector<uint8_t> scode, lc;
    for (int64_t c = 0; c < idx->K; ++c) {
        const int64_t n = idx->sizes[c], nb = (n + kBlock - 1) / kBlock, b0 = blk_off[c], v0 = vec_off[c];
        if (S > 1) {
            sfac.resize(64 * S * nb);
            r.read(sfac.data(), 4 * sfac.size());
        }
        scode.resize(z.block_bytes * nb);
        r.read(scode.data(), scode.size());
        int64_t lc_alloc = z.long_stride * n;
        if (S > 1 && idx->compact) {  // segment-major arrays rounded to 16 bytes (cluster_data.hpp:281-284)
            int64_t t = 0;
            for (size_t s = 0; s < S; ++s) t += (z.pv[s] * n + 15) / 16 * 16;
            lc_alloc = std::max(lc_alloc, t);
        }
        lc.assign(lc_alloc, 0);
        r.read(lc.data(), z.long_stride * n);
        lfac.resize(2 * S * n);
        r.read(lfac.data(), 4 * lfac.size());
        r.read(ids.data() + v0, 4 * n);
        for (size_t s = 0; s < S; ++s) r.read(rcent[s].data() + c * idx->segs[s].dim, 4 * idx->segs[s].dim);

        for (size_t s = 0; s < S; ++s) {
            const int64_t dim = idx->segs[s].dim, cols = dim / 8;
            for (int64_t b = 0; b < nb; ++b) {
                const float *fac = S == 1 ? reinterpret_cast<const float *>(scode.data() + b * z.block_bytes)
                                          : sfac.data() + (b * S + s) * 64;
                std::memcpy(&onorm[s][(b0 + b) * kBlock], fac, 4 * kBlock);
                std::memcpy(&ipc[s][(b0 + b) * kBlock], fac + kBlock, 4 * kBlock);
                if (!idx->segs[s].bits) continue;
                const uint8_t *blkp = scode.data() + b * z.block_bytes + (S == 1 ? 256 : z.scoff[s]);
                // invert fastscan::pack_codes (fastscan.hpp:75-112)
                uint8_t *dst = codes[s].data() + (b0 + b) * kBlock * cols;
                for (int64_t i = 0; i < cols; ++i)
                    for (int j = 0; j < 16; ++j) {
                        const uint8_t hi = blkp[i * 32 + j], lo = blkp[i * 32 + 16 + j];
                        const int v0l = kPerm0[j], v1l = kPerm0[j] + 16;
                        const uint8_t byte0 = (uint8_t)(((hi & 15) << 4) | (lo & 15));
                        const uint8_t byte1 = (uint8_t)(((hi >> 4) << 4) | (lo >> 4));
                        // [block][chunk of 8 bytes][lane][byte]
                        dst[((i / 8) * kBlock + v0l) * 8 + (i % 8)] = byte0;
                        dst[((i / 8) * kBlock + v1l) * 8 + (i % 8)] = byte1;
                    }
            }
            const int64_t ls = lstride_of(z.pv[s]);
            int64_t seg_base = 0;
            if (S > 1 && idx->compact)
                for (size_t t = 0; t < s; ++t) seg_base += (z.pv[t] * n + 15) / 16 * 16;
            for (int64_t v = 0; v < n; ++v) {
                const uint8_t *src = S == 1             ? lc.data() + v * z.pv[0]
                                     : idx->compact ? lc.data() + seg_base + v * z.pv[s]
                                                    : lc.data() + v * z.long_stride + z.loff[s];
                if (z.pv[s]) std::memcpy(&lcode[s][(v0 + v) * ls], src, z.pv[s]);
                exfac[s][2 * (v0 + v)] = lfac[(v * S + s) * 2];
                exfac[s][2 * (v0 + v) + 1] = lfac[(v * S + s) * 2 + 1];
            }
        }
    }
    uint8_t extra;
    if (std::fread(&extra, 1, 1, f) == 1) throw Error{SAQG_ERR_IO, "trailing bytes in index file " + path};
    return std::move(*idx);
}

// Device arrays from a host index (consumed).
Index *upload_index(HostIndex &&h) {
    auto idx = std::make_unique<Index>();
    cudaGetDevice(&idx->device);
    idx->N = h.N;
    idx->D = h.D;
    idx->K = h.K;
    std::memcpy(idx->qcfg_raw, h.qcfg_raw, 32);
    idx->var = std::move(h.var);
    idx->segs = std::move(h.segs);
    idx->compact = h.compact;
    idx->sizes = std::move(h.sizes);
    idx->blk_off.assign(idx->K + 1, 0);
    idx->vec_off.assign(idx->K + 1, 0);
    for (int64_t c = 0; c < idx->K; ++c) {
        idx->blk_off[c + 1] = idx->blk_off[c] + (idx->sizes[c] + kBlock - 1) / kBlock;
        idx->vec_off[c + 1] = idx->vec_off[c] + idx->sizes[c];
    }
    idx->total_blocks = idx->blk_off[idx->K];
    const int64_t N = idx->N;
    const SegSizes z = seg_sizes(idx->segs, idx->compact);
    const size_t S = idx->segs.size();
    int64_t dsum = 0;
    for (auto &sg : idx->segs) dsum += sg.dim;
    auto &cent = h.cent;
    auto &ids = h.ids;
    auto &codes = h.codes, &lcode = h.lcode;
    auto &onorm = h.onorm, &ipc = h.ipc, &rcent = h.rcent, &exfac = h.exfac;
    Index &I = *idx;
    DevIndexView &v = I.view;
    float *dcent = (float *)I.dalloc(4 * cent.size());
    I.upload(dcent, cent.data(), 4 * cent.size());
    v.centroids = dcent;
    std::vector<float> varp(dsum, 0.0f);
    std::memcpy(varp.data(), I.var.data(), 4 * std::min<int64_t>(dsum, (int64_t)I.var.size()));
    float *dvar = (float *)I.dalloc(4 * varp.size());
    I.upload(dvar, varp.data(), 4 * varp.size());
    v.var = dvar;
    uint32_t *dids = (uint32_t *)I.dalloc(4 * std::max<int64_t>(N, 1));
    I.upload(dids, ids.data(), 4 * N);
    v.ids = dids;
    int64_t *dbo = (int64_t *)I.dalloc(8 * (I.K + 1));
    I.upload(dbo, I.blk_off.data(), 8 * (I.K + 1));
    v.blk_off = dbo;
    int64_t *dvo = (int64_t *)I.dalloc(8 * (I.K + 1));
    I.upload(dvo, I.vec_off.data(), 8 * (I.K + 1));
    v.vec_off = dvo;
    for (size_t s = 0; s < S; ++s) {
        SegDev &g = v.seg[s];
        g.dim = (int)I.segs[s].dim;
        g.bits = (int)I.segs[s].bits;
        g.pv = (int)z.pv[s];
        g.lstride = (int)lstride_of(z.pv[s]);
        if (I.segs[s].rotated) {
            g.P = (float *)I.dalloc(4 * I.segs[s].P.size());
            I.upload(g.P, I.segs[s].P.data(), 4 * I.segs[s].P.size());
        }
        g.codes = (uint2 *)I.dalloc(codes[s].size());
        I.upload(g.codes, codes[s].data(), codes[s].size());
        g.onorm = (float *)I.dalloc(4 * onorm[s].size());
        I.upload(g.onorm, onorm[s].data(), 4 * onorm[s].size());
        g.ipcent = (float *)I.dalloc(4 * ipc[s].size());
        I.upload(g.ipcent, ipc[s].data(), 4 * ipc[s].size());
        g.lcode = (uint8_t *)I.dalloc(lcode[s].size());
        I.upload(g.lcode, lcode[s].data(), lcode[s].size());
        g.exfac = (float2 *)I.dalloc(4 * exfac[s].size());
        I.upload(g.exfac, exfac[s].data(), 4 * exfac[s].size());
        g.cent = (float *)I.dalloc(4 * rcent[s].size());
        I.upload(g.cent, rcent[s].data(), 4 * rcent[s].size());
    }
    finalize_view(I);
    return idx.release();
}

// Host copy of a device index.
HostIndex download_index(const Index &I) {
    HostIndex h;
    h.N = I.N;
    h.D = I.D;
    h.K = I.K;
    std::memcpy(h.qcfg_raw, I.qcfg_raw, 32);
    h.var = I.var;
    h.segs = I.segs;
    h.compact = I.compact;
    h.sizes = I.sizes;
    const size_t S = I.segs.size();
    const int64_t N = I.N, NB = I.total_blocks;
    auto down = [](void *dst, const void *src, size_t bytes) {
        if (bytes) SAQG_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    };
    auto &cent = h.cent;
    cent.resize(I.K * I.D);
    down(cent.data(), I.view.centroids, 4 * cent.size());
    auto &ids = h.ids;
    ids.resize(N);
    down(ids.data(), I.view.ids, 4 * N);
    auto &codes = h.codes, &lcode = h.lcode;
    auto &onorm = h.onorm, &ipc = h.ipc, &rcent = h.rcent, &exfac = h.exfac;
    codes.resize(S);
    lcode.resize(S);
    onorm.resize(S);
    ipc.resize(S);
    rcent.resize(S);
    exfac.resize(S);
    for (size_t s = 0; s < S; ++s) {
        const SegDev &g = I.view.seg[s];
        codes[s].resize(g.bits ? NB * kBlock * g.dim / 8 : 0);
        down(codes[s].data(), g.codes, codes[s].size());
        onorm[s].resize(NB * kBlock);
        down(onorm[s].data(), g.onorm, 4 * onorm[s].size());
        ipc[s].resize(NB * kBlock);
        down(ipc[s].data(), g.ipcent, 4 * ipc[s].size());
        lcode[s].resize((size_t)N * g.lstride);
        down(lcode[s].data(), g.lcode, lcode[s].size());
        exfac[s].resize(2 * N);
        down(exfac[s].data(), g.exfac, 4 * exfac[s].size());
        rcent[s].resize(I.K * g.dim);
        down(rcent[s].data(), g.cent, 4 * rcent[s].size());
    }
    return h;
}

// Reference file (IVF::save, ivf.hpp:197-228) from a host index.
void write_reference(const HostIndex &h, const std::string &path) {
    const size_t S = h.segs.size();
    const SegSizes z = seg_sizes(h.segs, h.compact);
    const int64_t N = h.N;
    std::vector<int64_t> blk_off(h.K + 1, 0), vec_off(h.K + 1, 0);
    for (int64_t c = 0; c < h.K; ++c) {
        blk_off[c + 1] = blk_off[c] + (h.sizes[c] + kBlock - 1) / kBlock;
        vec_off[c + 1] = vec_off[c] + h.sizes[c];
    }
    const auto &cent = h.cent;
    const auto &ids = h.ids;
    const auto &codes = h.codes, &lcode = h.lcode;
    const auto &onorm = h.onorm, &ipc = h.ipc, &rcent = h.rcent, &exfac = h.exfac;
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) throw Error{SAQG_ERR_IO, "cannot write " + path};
    std::unique_ptr<FILE, int (*)(FILE *)> guard(f, std::fclose);
    auto w = [&](const void *p, size_t n) {
        if (n && std::fwrite(p, 1, n, f) != n) throw Error{SAQG_ERR_IO, "write failed: " + path};
    };
    auto w64 = [&](uint64_t v) { w(&v, 8); };
    w64(N);
    w64(h.D);
    w64(h.K);
    w(cent.data(), 4 * cent.size());
    w(h.qcfg_raw, 32);
    w64(h.D);
    w64(h.var.size());
    w(h.var.data(), 4 * h.var.size());
    w64(S);
    for (auto &sg : h.segs) {
        w64(sg.dim);
        w64(sg.bits);
        w(sg.cfg_raw, 20);
        uint8_t flag = sg.rotated ? 1 : 0;
        w(&flag, 1);
        if (sg.rotated) w(sg.P.data(), 4 * sg.P.size());
    }
    w(h.sizes.data(), 8 * h.K);
    std::vector<float> sfac;
    std::vector<uint8_t> scode, lc;
    std::vector<float> lfac;
    for (int64_t c = 0; c < h.K; ++c) {
        const int64_t n = h.sizes[c], nb = (n + kBlock - 1) / kBlock, b0 = blk_off[c], v0 = vec_off[c];
        sfac.assign(S > 1 ? 64 * S * nb : 0, 0.0f);
        scode.assign(z.block_bytes * nb, 0);
        for (size_t s = 0; s < S; ++s) {
            const int64_t dim = h.segs[s].dim, cols = dim / 8;
            for (int64_t b = 0; b < nb; ++b) {
                float *fac = S == 1 ? reinterpret_cast<float *>(scode.data() + b * z.block_bytes)
                                    : sfac.data() + (b * S + s) * 64;
                std::memcpy(fac, &onorm[s][(b0 + b) * kBlock], 4 * kBlock);
                std::memcpy(fac + kBlock, &ipc[s][(b0 + b) * kBlock], 4 * kBlock);
                if (!h.segs[s].bits) continue;
                uint8_t *blkp = scode.data() + b * z.block_bytes + (S == 1 ? 256 : z.scoff[s]);
                const uint8_t *src = codes[s].data() + (b0 + b) * kBlock * cols;
                for (int64_t i = 0; i < cols; ++i)
                    for (int j = 0; j < 16; ++j) {
                        const uint8_t byte0 = src[((i / 8) * kBlock + kPerm0[j]) * 8 + (i % 8)];
                        const uint8_t byte1 = src[((i / 8) * kBlock + kPerm0[j] + 16) * 8 + (i % 8)];
                        blkp[i * 32 + j] = (uint8_t)((byte0 >> 4) | ((byte1 >> 4) << 4));
                        blkp[i * 32 + 16 + j] = (uint8_t)((byte0 & 15) | ((byte1 & 15) << 4));
                    }
            }
        }
        lc.assign(z.long_stride * n, 0);
        lfac.assign(2 * S * n, 0.0f);
        for (size_t s = 0; s < S; ++s) {
            int64_t seg_base = 0;
            if (S > 1 && h.compact)
                for (size_t t = 0; t < s; ++t) seg_base += (z.pv[t] * n + 15) / 16 * 16;
            const int64_t ls = lstride_of(z.pv[s]);
            for (int64_t v = 0; v < n; ++v) {
                int64_t off = S == 1 ? v * z.pv[0] : h.compact ? seg_base + v * z.pv[s] : v * z.long_stride + z.loff[s];
                if (z.pv[s] && off + z.pv[s] <= (int64_t)lc.size())
                    std::memcpy(lc.data() + off, &lcode[s][(v0 + v) * ls], z.pv[s]);
                lfac[(v * S + s) * 2] = exfac[s][2 * (v0 + v)];
                lfac[(v * S + s) * 2 + 1] = exfac[s][2 * (v0 + v) + 1];
            }
        }
        if (S > 1) w(sfac.data(), 4 * sfac.size());
        w(scode.data(), scode.size());
        w(lc.data(), lc.size());
        w(lfac.data(), 4 * lfac.size());
        w(ids.data() + v0, 4 * n);
        for (size_t s = 0; s < S; ++s) w(rcent[s].data() + c * h.segs[s].dim, 4 * h.segs[s].dim);
    }
}


// ------------------------------------------------------------ format v2
// A versioned, checksummed file holding the device layout as-is, each array
// at a 4096-byte aligned offset, so loading is a read and a copy per array:
//   header: magic "SAQGIDX2", u32 version (2), u32 header bytes, u64 N, D, K,
//     #segments, compact flag, #variance values, QuantizeConfig (32 raw
//     bytes); per segment: u64 dim, bits; QuantSingleConfig (20 raw bytes),
//     u8 rotated, 3 zero bytes; u64 #sections; per section: u32 kind, u32
//     segment, u64 offset, u64 bytes, u64 checksum; u64 checksum of the header
//     up to here.
//   sections: 1 centroids [K][D] f32, 2 variance f32, 3 cluster sizes [K] i64,
//     4 ids [N] u32; per segment 10 P [dim][dim] f32 (rotated segments),
//     11 1-bit codes [block][dim/64][32] x 8 bytes, 12 |o| [block][32] f32,
//     13 ip_cent_oa [block][32] f32, 14 ex-codes [N][row padded to 16 bytes],
//     15 ex factors [N] (rescale, error) f32, 16 rotated centroids [K][dim] f32.
// Checksum: 64-bit FNV-1a over 8-byte little-endian words, the tail padded
// with zero bytes.
namespace {
const char kMagicV2[8] = {'S', 'A', 'Q', 'G', 'I', 'D', 'X', '2'};
constexpr uint32_t kVersionV2 = 2;
constexpr uint64_t kAlignV2 = 4096;

uint64_t checksum64(const void *data, size_t n) {
    const uint8_t *p = static_cast<const uint8_t *>(data);
    uint64_t h = 1469598103934665603ull;
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
        uint64_t w;
        std::memcpy(&w, p + i, 8);
        h = (h ^ w) * 1099511628211ull;
    }
    if (i < n) {
        uint64_t w = 0;
        std::memcpy(&w, p + i, n - i);
        h = (h ^ w) * 1099511628211ull;
    }
    return h;
}

struct SectionV2 {
    uint32_t kind, seg;
    uint64_t offset, bytes, sum;
};

struct ByteWriter {
    std::vector<uint8_t> b;
    void put(const void *p, size_t n) {
        const uint8_t *c = static_cast<const uint8_t *>(p);
        b.insert(b.end(), c, c + n);
    }
    void u32(uint32_t v) { put(&v, 4); }
    void u64(uint64_t v) { put(&v, 8); }
};

struct ByteReader {
    const uint8_t *p;
    size_t n, at = 0;
    std::string path;
    void get(void *dst, size_t k) {
        if (at + k > n) throw Error{SAQG_ERR_IO, "truncated header in " + path};
        std::memcpy(dst, p + at, k);
        at += k;
    }
    uint32_t u32() {
        uint32_t v;
        get(&v, 4);
        return v;
    }
    uint64_t u64() {
        uint64_t v;
        get(&v, 8);
        return v;
    }
};
}  // namespace

bool is_v2_file(const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) throw Error{SAQG_ERR_IO, "cannot open index file " + path};
    char m[8] = {0};
    const size_t got = std::fread(m, 1, 8, f);
    std::fclose(f);
    return got == 8 && std::memcmp(m, kMagicV2, 8) == 0;
}

void write_v2(const HostIndex &h, const std::string &path) {
    struct Piece {
        uint32_t kind, seg;
        const void *data;
        uint64_t bytes;
    };
    std::vector<Piece> pieces;
    pieces.push_back({1, 0, h.cent.data(), 4 * (uint64_t)h.cent.size()});
    pieces.push_back({2, 0, h.var.data(), 4 * (uint64_t)h.var.size()});
    pieces.push_back({3, 0, h.sizes.data(), 8 * (uint64_t)h.sizes.size()});
    pieces.push_back({4, 0, h.ids.data(), 4 * (uint64_t)h.ids.size()});
    for (uint32_t s = 0; s < h.segs.size(); ++s) {
        if (h.segs[s].rotated) pieces.push_back({10, s, h.segs[s].P.data(), 4 * (uint64_t)h.segs[s].P.size()});
        pieces.push_back({11, s, h.codes[s].data(), (uint64_t)h.codes[s].size()});
        pieces.push_back({12, s, h.onorm[s].data(), 4 * (uint64_t)h.onorm[s].size()});
        pieces.push_back({13, s, h.ipc[s].data(), 4 * (uint64_t)h.ipc[s].size()});
        pieces.push_back({14, s, h.lcode[s].data(), (uint64_t)h.lcode[s].size()});
        pieces.push_back({15, s, h.exfac[s].data(), 4 * (uint64_t)h.exfac[s].size()});
        pieces.push_back({16, s, h.rcent[s].data(), 4 * (uint64_t)h.rcent[s].size()});
    }
    // header size is known before the offsets: fixed part + segments + section table + checksum
    const uint64_t hdr_bytes = 8 + 4 + 4 + 6 * 8 + 32 + h.segs.size() * (16 + 20 + 4) + 8 + pieces.size() * 32 + 8;
    uint64_t off = (hdr_bytes + kAlignV2 - 1) / kAlignV2 * kAlignV2;
    std::vector<SectionV2> secs;
    for (auto &pc : pieces) {
        secs.push_back({pc.kind, pc.seg, off, pc.bytes, checksum64(pc.data, pc.bytes)});
        off += (pc.bytes + kAlignV2 - 1) / kAlignV2 * kAlignV2;
    }
    ByteWriter w;
    w.put(kMagicV2, 8);
    w.u32(kVersionV2);
    w.u32((uint32_t)hdr_bytes);
    w.u64(h.N);
    w.u64(h.D);
    w.u64(h.K);
    w.u64(h.segs.size());
    w.u64(h.compact ? 1 : 0);
    w.u64(h.var.size());
    w.put(h.qcfg_raw, 32);
    for (auto &sg : h.segs) {
        w.u64(sg.dim);
        w.u64(sg.bits);
        w.put(sg.cfg_raw, 20);
        const uint8_t tail[4] = {(uint8_t)(sg.rotated ? 1 : 0), 0, 0, 0};
        w.put(tail, 4);
    }
    w.u64(secs.size());
    for (auto &sc : secs) {
        w.u32(sc.kind);
        w.u32(sc.seg);
        w.u64(sc.offset);
        w.u64(sc.bytes);
        w.u64(sc.sum);
    }
    w.u64(checksum64(w.b.data(), w.b.size()));
    if (w.b.size() != hdr_bytes) throw Error{SAQG_ERR_INTERNAL, "v2 header size mismatch"};
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) throw Error{SAQG_ERR_IO, "cannot write " + path};
    std::unique_ptr<FILE, int (*)(FILE *)> guard(f, std::fclose);
    auto put = [&](const void *p, size_t n) {
        if (n && std::fwrite(p, 1, n, f) != n) throw Error{SAQG_ERR_IO, "write failed: " + path};
    };
    put(w.b.data(), w.b.size());
    uint64_t at = w.b.size();
    static const std::vector<uint8_t> zeros(kAlignV2, 0);
    for (size_t i = 0; i < pieces.size(); ++i) {
        if (secs[i].offset > at) put(zeros.data(), secs[i].offset - at);
        put(pieces[i].data, pieces[i].bytes);
        at = secs[i].offset + pieces[i].bytes;
    }
    const uint64_t end = (at + kAlignV2 - 1) / kAlignV2 * kAlignV2;
    if (end > at) put(zeros.data(), end - at);
}

HostIndex parse_v2(const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) throw Error{SAQG_ERR_IO, "cannot open index file " + path};
    std::unique_ptr<FILE, int (*)(FILE *)> guard(f, std::fclose);
    uint8_t fixed[16];
    if (std::fread(fixed, 1, 16, f) != 16 || std::memcmp(fixed, kMagicV2, 8) != 0)
        throw Error{SAQG_ERR_IO, "not a v2 index file: " + path};
    uint32_t version, hdr_bytes;
    std::memcpy(&version, fixed + 8, 4);
    std::memcpy(&hdr_bytes, fixed + 12, 4);
    if (version != kVersionV2) throw Error{SAQG_ERR_IO, "unsupported v2 index version in " + path};
    if (hdr_bytes < 16 + 8 || hdr_bytes > (1u << 24)) throw Error{SAQG_ERR_IO, "implausible v2 header in " + path};
    std::vector<uint8_t> hdr(hdr_bytes);
    std::memcpy(hdr.data(), fixed, 16);
    if (std::fread(hdr.data() + 16, 1, hdr_bytes - 16, f) != hdr_bytes - 16)
        throw Error{SAQG_ERR_IO, "truncated v2 header in " + path};
    uint64_t want;
    std::memcpy(&want, hdr.data() + hdr_bytes - 8, 8);
    if (checksum64(hdr.data(), hdr_bytes - 8) != want) throw Error{SAQG_ERR_IO, "v2 header checksum mismatch in " + path};
    ByteReader r{hdr.data(), hdr_bytes - 8, 16, path};
    HostIndex h;
    h.N = (int64_t)r.u64();
    h.D = (int64_t)r.u64();
    h.K = (int64_t)r.u64();
    const uint64_t S = r.u64();
    h.compact = r.u64() != 0;
    const uint64_t nvar = r.u64();
    r.get(h.qcfg_raw, 32);
    if (h.D <= 0 || h.K <= 0 || h.N < 0 || h.D > (1 << 20) || h.K > (1 << 28) || S < 1 || S > (uint64_t)kMaxSeg ||
        nvar != (uint64_t)h.D)
        throw Error{SAQG_ERR_IO, "implausible v2 header in " + path};
    for (uint64_t s = 0; s < S; ++s) {
        Index::SegHost sg;
        sg.dim = (int64_t)r.u64();
        sg.bits = (int64_t)r.u64();
        r.get(sg.cfg_raw, 20);
        uint8_t tail[4];
        r.get(tail, 4);
        sg.rotated = tail[0] != 0;
        if (sg.dim <= 0 || sg.dim % 64 || sg.bits > kMaxBits || sg.dim > 16384)
            throw Error{SAQG_ERR_IO, "unsupported segment in " + path};
        h.segs.push_back(std::move(sg));
    }
    const uint64_t nsec = r.u64();
    if (nsec > 4 + 7 * S) throw Error{SAQG_ERR_IO, "implausible v2 section table in " + path};
    std::vector<SectionV2> secs(nsec);
    for (auto &sc : secs) {
        sc.kind = r.u32();
        sc.seg = r.u32();
        sc.offset = r.u64();
        sc.bytes = r.u64();
        sc.sum = r.u64();
        if (sc.seg >= S) throw Error{SAQG_ERR_IO, "bad v2 section in " + path};
    }
    // sizes first: they fix every other array's length
    std::vector<int64_t> blk_off(h.K + 1, 0);
    h.codes.resize(S);
    h.lcode.resize(S);
    h.onorm.resize(S);
    h.ipc.resize(S);
    h.rcent.resize(S);
    h.exfac.resize(S);
    auto load = [&](const SectionV2 &sc, void *dst, uint64_t expect) {
        if (sc.bytes != expect) throw Error{SAQG_ERR_IO, "v2 section size mismatch in " + path};
        if (!expect) return;
        if (std::fseek(f, (long)sc.offset, SEEK_SET) != 0 || std::fread(dst, 1, expect, f) != expect)
            throw Error{SAQG_ERR_IO, "truncated v2 section in " + path};
        if (checksum64(dst, expect) != sc.sum) throw Error{SAQG_ERR_IO, "v2 section checksum mismatch in " + path};
    };
    auto find = [&](uint32_t kind, uint32_t seg) -> const SectionV2 * {
        for (auto &sc : secs)
            if (sc.kind == kind && sc.seg == seg) return &sc;
        return nullptr;
    };
    auto need = [&](uint32_t kind, uint32_t seg) -> const SectionV2 & {
        const SectionV2 *sc = find(kind, seg);
        if (!sc) throw Error{SAQG_ERR_IO, "missing v2 section in " + path};
        return *sc;
    };
    h.sizes.resize(h.K);
    load(need(3, 0), h.sizes.data(), 8 * (uint64_t)h.K);
    int64_t total = 0;
    for (int64_t c = 0; c < h.K; ++c) {
        if (h.sizes[c] < 0) throw Error{SAQG_ERR_IO, "negative cluster size in " + path};
        blk_off[c + 1] = blk_off[c] + (h.sizes[c] + kBlock - 1) / kBlock;
        total += h.sizes[c];
    }
    if (total != h.N) throw Error{SAQG_ERR_IO, "cluster sizes do not sum to N in " + path};
    const int64_t NB = blk_off[h.K];
    const SegSizes z = seg_sizes(h.segs, h.compact);
    h.cent.resize(h.K * h.D);
    load(need(1, 0), h.cent.data(), 4 * (uint64_t)h.cent.size());
    h.var.resize(nvar);
    load(need(2, 0), h.var.data(), 4 * nvar);
    h.ids.resize(h.N);
    load(need(4, 0), h.ids.data(), 4 * (uint64_t)h.N);
    for (uint32_t s = 0; s < S; ++s) {
        auto &sg = h.segs[s];
        if (sg.rotated) {
            sg.P.resize(sg.dim * sg.dim);
            load(need(10, s), sg.P.data(), 4 * (uint64_t)sg.P.size());
        } else if (find(10, s)) {
            throw Error{SAQG_ERR_IO, "unexpected rotation in " + path};
        }
        h.codes[s].resize(sg.bits ? NB * kBlock * sg.dim / 8 : 0);
        load(need(11, s), h.codes[s].data(), h.codes[s].size());
        h.onorm[s].resize(NB * kBlock);
        load(need(12, s), h.onorm[s].data(), 4 * (uint64_t)h.onorm[s].size());
        h.ipc[s].resize(NB * kBlock);
        load(need(13, s), h.ipc[s].data(), 4 * (uint64_t)h.ipc[s].size());
        h.lcode[s].resize((size_t)h.N * lstride_of(z.pv[s]));
        load(need(14, s), h.lcode[s].data(), h.lcode[s].size());
        h.exfac[s].resize(2 * h.N);
        load(need(15, s), h.exfac[s].data(), 4 * (uint64_t)h.exfac[s].size());
        h.rcent[s].resize(h.K * sg.dim);
        load(need(16, s), h.rcent[s].data(), 4 * (uint64_t)h.rcent[s].size());
    }
    int64_t dsum = 0;
    for (auto &sg : h.segs) dsum += sg.dim;
    if (dsum < h.D || h.D % 64 != 0) throw Error{SAQG_ERR_IO, "dimension must be a multiple of 64 in " + path};
    return h;
}

Index *load_index_file(const std::string &path) {
    return upload_index(is_v2_file(path) ? parse_v2(path) : parse_reference(path));
}

void save_index_file(const Index &I, const std::string &path) { write_reference(download_index(I), path); }

void save_index_v2(const Index &I, const std::string &path) { write_v2(download_index(I), path); }

void convert_index_file(const std::string &src, const std::string &dst, int format) {
    HostIndex h = is_v2_file(src) ? parse_v2(src) : parse_reference(src);
    if (format == SAQG_FORMAT_V2) write_v2(h, dst);
    else write_reference(h, dst);
}

}  // namespace saqg
