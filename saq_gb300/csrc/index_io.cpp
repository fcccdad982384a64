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

#include <cublas_v2.h>

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

SegSizes seg_sizes(const Index &idx) {
    SegSizes z;
    const size_t S = idx.segs.size();
    z.sc.resize(S);
    z.pv.resize(S);
    z.loff.resize(S);
    z.scoff.resize(S);
    for (size_t s = 0; s < S; ++s) {
        z.sc[s] = idx.segs[s].bits ? idx.segs[s].dim * kBlock / 8 : 0;
        z.pv[s] = idx.segs[s].bits ? idx.segs[s].dim * (idx.segs[s].bits - 1) / 8 : 0;
    }
    if (S == 1) {
        z.block_bytes = 64 * 4 + z.sc[0];
        z.long_stride = z.pv[0];
    } else {
        for (size_t s = 0; s < S; ++s) {
            z.scoff[s] = z.block_bytes;
            z.block_bytes += z.sc[s];
            z.loff[s] = z.long_stride;
            z.long_stride += idx.compact ? z.pv[s] : (z.pv[s] + 15) / 16 * 16;
        }
    }
    return z;
}

int64_t lstride_of(int64_t pv) { return (pv + 15) / 16 * 16; }
}  // namespace

Index::~Index() {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(device);
    for (void *p : allocations) cudaFree(p);
    if (scratch) cudaFree(scratch);
    if (split_scratch) cudaFree(split_scratch);
    if (aux) cudaStreamDestroy(aux);
    if (cnorm2) cudaFree(cnorm2);
    if (blas) cublasDestroy(static_cast<cublasHandle_t>(blas));
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    cudaSetDevice(cur);
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

void *Index::split_scratch_get(size_t bytes) const { return grow(split_scratch, split_scratch_bytes, bytes); }

// The split pass is a batch's critical path: its stream gets the device's
// highest priority, so its CTAs go first while the CTA scan beside it fills in.
cudaStream_t Index::aux_stream() const {
    if (!aux) {
        int least = 0, greatest = 0;
        SAQG_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        SAQG_CUDA_TRY(cudaStreamCreateWithPriority(&aux, cudaStreamNonBlocking, greatest));
    }
    return aux;
}
cudaEvent_t Index::fork_event() const {
    if (!ev_fork) SAQG_CUDA_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    return ev_fork;
}
cudaEvent_t Index::join_event() const {
    if (!ev_join) SAQG_CUDA_TRY(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    return ev_join;
}

void *Index::scratch_get(size_t bytes) const {
    if (bytes > scratch_bytes) {
        SAQG_CUDA_TRY(cudaDeviceSynchronize());
        if (scratch) SAQG_CUDA_TRY(cudaFree(scratch));
        scratch = nullptr;
        scratch_bytes = 0;
        size_t want = bytes + bytes / 4 + (1 << 20);
        cudaError_t e = cudaMalloc(&scratch, want);
        if (e != cudaSuccess) throw Error{SAQG_ERR_NOMEM, std::string("scratch cudaMalloc failed: ") + cudaGetErrorString(e)};
        scratch_bytes = want;
    }
    return scratch;
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

Index *load_index_file(const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) throw Error{SAQG_ERR_IO, "cannot open index file " + path};
    std::unique_ptr<FILE, int (*)(FILE *)> guard(f, std::fclose);
    Reader r{f, path};
    auto idx = std::make_unique<Index>();
    cudaGetDevice(&idx->device);
    idx->N = (int64_t)r.u64();
    idx->D = (int64_t)r.u64();
    idx->K = (int64_t)r.u64();
    if (idx->D <= 0 || idx->K <= 0 || idx->N < 0 || idx->D > (1 << 20) || idx->K > (1 << 28))
        throw Error{SAQG_ERR_IO, "implausible header in " + path};
    std::vector<float> cent(idx->K * idx->D);
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
    idx->blk_off.assign(idx->K + 1, 0);
    idx->vec_off.assign(idx->K + 1, 0);
    for (int64_t c = 0; c < idx->K; ++c) {
        idx->blk_off[c + 1] = idx->blk_off[c] + (idx->sizes[c] + kBlock - 1) / kBlock;
        idx->vec_off[c + 1] = idx->vec_off[c] + idx->sizes[c];
    }
    if (idx->vec_off[idx->K] != idx->N) throw Error{SAQG_ERR_IO, "cluster sizes do not sum to N in " + path};
    const int64_t NB = idx->blk_off[idx->K], N = idx->N;
    idx->total_blocks = NB;
    const SegSizes z = seg_sizes(*idx);
    const size_t S = idx->segs.size();

    // host staging of the device layout
    std::vector<std::vector<uint8_t>> codes(S), lcode(S);
    std::vector<std::vector<float>> onorm(S), ipc(S), rcent(S);
    std::vector<std::vector<float>> exfac(S);
    for (size_t s = 0; s < S; ++s) {
        const int64_t dim = idx->segs[s].dim;
        codes[s].assign(idx->segs[s].bits ? NB * kBlock * dim / 8 : 0, 0);
        onorm[s].assign(NB * kBlock, 0.0f);
        ipc[s].assign(NB * kBlock, 0.0f);
        lcode[s].assign(N * lstride_of(z.pv[s]), 0);
        exfac[s].assign(2 * N, 0.0f);
        rcent[s].assign(idx->K * dim, 0.0f);
    }
    std::vector<uint32_t> ids(N);
    std::vector<float> sfac, blk, lfac;
    std::vector<uint8_t> scode, lc;
    for (int64_t c = 0; c < idx->K; ++c) {
        const int64_t n = idx->sizes[c], nb = (n + kBlock - 1) / kBlock, b0 = idx->blk_off[c], v0 = idx->vec_off[c];
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

    // upload
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

// Device layout -> reference file (IVF::save, ivf.hpp:197-228).
void save_index_file(const Index &I, const std::string &path) {
    const size_t S = I.segs.size();
    const int64_t N = I.N, NB = I.total_blocks;
    const SegSizes z = seg_sizes(I);
    auto down = [](void *dst, const void *src, size_t bytes) {
        if (bytes) SAQG_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    };
    std::vector<float> cent(I.K * I.D);
    down(cent.data(), I.view.centroids, 4 * cent.size());
    std::vector<uint32_t> ids(N);
    down(ids.data(), I.view.ids, 4 * N);
    std::vector<std::vector<uint8_t>> codes(S), lcode(S);
    std::vector<std::vector<float>> onorm(S), ipc(S), rcent(S), exfac(S);
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
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) throw Error{SAQG_ERR_IO, "cannot write " + path};
    std::unique_ptr<FILE, int (*)(FILE *)> guard(f, std::fclose);
    auto w = [&](const void *p, size_t n) {
        if (n && std::fwrite(p, 1, n, f) != n) throw Error{SAQG_ERR_IO, "write failed: " + path};
    };
    auto w64 = [&](uint64_t v) { w(&v, 8); };
    w64(N);
    w64(I.D);
    w64(I.K);
    w(cent.data(), 4 * cent.size());
    w(I.qcfg_raw, 32);
    w64(I.D);
    w64(I.var.size());
    w(I.var.data(), 4 * I.var.size());
    w64(S);
    for (auto &sg : I.segs) {
        w64(sg.dim);
        w64(sg.bits);
        w(sg.cfg_raw, 20);
        uint8_t flag = sg.rotated ? 1 : 0;
        w(&flag, 1);
        if (sg.rotated) w(sg.P.data(), 4 * sg.P.size());
    }
    w(I.sizes.data(), 8 * I.K);
    std::vector<float> sfac;
    std::vector<uint8_t> scode, lc;
    std::vector<float> lfac;
    for (int64_t c = 0; c < I.K; ++c) {
        const int64_t n = I.sizes[c], nb = (n + kBlock - 1) / kBlock, b0 = I.blk_off[c], v0 = I.vec_off[c];
        sfac.assign(S > 1 ? 64 * S * nb : 0, 0.0f);
        scode.assign(z.block_bytes * nb, 0);
        for (size_t s = 0; s < S; ++s) {
            const int64_t dim = I.segs[s].dim, cols = dim / 8;
            for (int64_t b = 0; b < nb; ++b) {
                float *fac = S == 1 ? reinterpret_cast<float *>(scode.data() + b * z.block_bytes)
                                    : sfac.data() + (b * S + s) * 64;
                std::memcpy(fac, &onorm[s][(b0 + b) * kBlock], 4 * kBlock);
                std::memcpy(fac + kBlock, &ipc[s][(b0 + b) * kBlock], 4 * kBlock);
                if (!I.segs[s].bits) continue;
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
            if (S > 1 && I.compact)
                for (size_t t = 0; t < s; ++t) seg_base += (z.pv[t] * n + 15) / 16 * 16;
            const int64_t ls = lstride_of(z.pv[s]);
            for (int64_t v = 0; v < n; ++v) {
                int64_t off = S == 1 ? v * z.pv[0] : I.compact ? seg_base + v * z.pv[s] : v * z.long_stride + z.loff[s];
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
        for (size_t s = 0; s < S; ++s) w(rcent[s].data() + c * I.segs[s].dim, 4 * I.segs[s].dim);
    }
}

}  // namespace saqg
