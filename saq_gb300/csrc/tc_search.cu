// Tensor-core form of the batched search (no counterpart in the reference,
// whose search is one query at a time on AVX-512).
//
// For a batch of queries the quantized codes of every probed cluster are
// contracted with the queries that probe it as one dense product on the
// 5th-generation tensor cores:
//
//   approx(q, o) = sum_s |o_s|^2 + |r_s|^2 - 2 rescale_s (delta_s <r_s, u_s> + (delta_s/2 - 1) sum(r_s))
//
// where r_s = q_s P_s - c_s P_s is the query's rotated residual on segment s,
// u_s the vector's full B-bit CAQ code (1-bit part << (B-1) | ex-code) and
// delta_s = 2 / 2^B: CaqCluEstimator::compAccurateDist (caq_estimator.hpp:190-217)
// with the FastScan LUT of the 1-bit part replaced by the exact code.  Codes are
// held as BF16 (integers below 2^8 are exact), queries are rounded to BF16,
// products accumulate in FP32 in tensor memory.  The `shortlist` smallest
// approximate distances of each query are then re-ranked with the distance the
// exact search computes (k_tc_rerank), and the top-k of those is the answer.
//
// Kernels, in launch order:
//   k_tc_codes     (once per index) BF16 code matrix [vector][dim], clusters concatenated
//   k_tc_pairs     per-query candidate offsets (probe order) and per-cluster pair counts
//   k_excl_scan    exclusive prefix sums (query offsets, cluster bucket offsets)
//   k_tc_fill / k_tc_sort   pairs bucketed by cluster, each bucket in pair order
//   k_tc_gather    BF16 residual query row of every pair (cluster order), with
//                  its per-segment sum and squared norm
//   k_tc_contract  persistent, one CTA per SM over the 128-vector tiles of the
//                  clusters: TMA streams the code tile and the chunk's query rows
//                  through a 6-stage shared-memory ring (128-byte swizzle), one
//                  thread issues tcgen05.mma (M=128, N=pairs, K=16 per instruction)
//                  into per-segment TMEM accumulators (two, alternating by chunk),
//                  four warps read them back with tcgen05.ld for the epilogue
//   k_tc_select1/2 per query: the shortlist by radix select over 4,096-candidate
//                  chunks, then over the chunks' survivors, in candidate order
//   k_tc_groups / k_tc_rerank / k_tc_topk  (search.cu) exact distances of the
//                  shortlist, one CTA per (query, probed cluster), then top-k
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "saqg_internal.h"
#include "tcgen05.cuh"

namespace saqg {

namespace {

using namespace tc;

constexpr int kTcBM = 128;           // vectors per tile: the MMA's M
constexpr int kTcBK = 64;            // dims per pipeline stage: one 128-byte BF16 row
constexpr int kTcStages = 6;         // ring depth (one persistent CTA per SM)
constexpr int kTcThreads = 192;      // warp 0 TMA, warp 1 MMA + TMEM owner, warps 2-5 queries + epilogue
constexpr int kTcStageBytes = 16384; // 128 rows x 128 bytes (A), at most 128 x 128 bytes (B)
constexpr int kTcCols = 256;         // TMEM columns of one accumulator (segments x pairs per chunk); a CTA holds two
constexpr int kTcMaxN = 128;         // pairs per chunk at most (the MMA's N)
constexpr int kTcMaxShort = 1024;    // shortlist length at most
constexpr int kTcMaxBatch = 8192;    // queries per call at most (bucket sort in shared memory)

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M = 128, N = n.
__device__ __forceinline__ uint32_t idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTcBM >> 4) << 24);
}

// ------------------------------------------------------------ code matrix
// Value of dimension d of an ex-code of `b` bits in the reference's compacted
// layouts (CodeHelper<B>::compacted_code8/16, code_helper.hpp).
__device__ __forceinline__ uint32_t ex_bits8(const uint8_t *__restrict__ y, int D, int b, int d) {
    switch (b) {
    case 1:
        return (y[d >> 3] >> (d & 7)) & 1u;
    case 2:
    case 3: {
        const uint8_t *g = y + (d >> 6) * (b == 2 ? 16 : 24);
        const int k = d & 63;
        uint32_t v = (g[k & 15] >> (2 * (k >> 4))) & 3u;
        if (b == 3) v |= ((g[16 + (k & 7)] >> (k >> 3)) & 1u) << 2;
        return v;
    }
    case 4: {
        const uint8_t *g = y + (d >> 5) * 16;
        const int k = d & 31;
        return k < 16 ? (g[k] & 15u) : (uint32_t)(g[k - 16] >> 4);
    }
    case 5:
        return (ex_bits8(y, D, 4, d) << 1) | ex_bits8(y + D / 2, D, 1, d);
    case 6:
    case 7: {
        const uint8_t *g = y + (d >> 6) * (b == 6 ? 48 : 56);
        const int k = d & 63, r = k & 15;
        uint32_t v;
        if (k < 16) v = g[r] & 63u;
        else if (k < 32) v = g[16 + r] & 63u;
        else if (k < 48) v = ((uint32_t)(g[r] >> 6) << 4) | (g[32 + r] & 15u);
        else v = ((uint32_t)(g[16 + r] >> 6) << 4) | (uint32_t)(g[32 + r] >> 4);
        if (b == 7) v |= ((g[48 + (k & 7)] >> (k >> 3)) & 1u) << 6;
        return v;
    }
    case 8:
        return y[d];
    default:
        return 0;
    }
}

__device__ __forceinline__ uint32_t ex_value(const uint8_t *__restrict__ y, int D, int exb, int d) {
    if (exb > 8) return y[d] | (ex_bits8(y + D, D, exb - 8, d) << 8);
    return ex_bits8(y, D, exb, d);
}

// Full CAQ code u = (1-bit code << (B-1)) | ex-code of every vector, as BF16,
// row-major [vector][Dtot] (segments at their query offsets).  One thread per
// (vector, 8 dims).
__global__ void k_tc_codes(DevIndexView ix, const int32_t *__restrict__ cl_of, int64_t n, __nv_bfloat16 *__restrict__ A) {
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int per = ix.Dtot / 8;
    if (gid >= n * per) return;
    const int64_t v = gid / per;
    const int k8 = (int)(gid - v * per) * 8;
    int s = 0;
    while (s + 1 < ix.S && k8 >= ix.seg[s + 1].qoff) ++s;
    const SegDev &g = ix.seg[s];
    const int d0 = k8 - g.qoff;
    const int c = cl_of[v];
    const int64_t pos = v - ix.vec_off[c];
    const int64_t gb = ix.blk_off[c] + pos / 32;
    const int lane = (int)(pos % 32);
    const uint8_t *cb = reinterpret_cast<const uint8_t *>(g.codes) + (size_t)gb * (g.dim / 8) * 32;
    const int i = d0 / 8;
    const uint32_t msb = cb[((size_t)(i / 8) * 32 + lane) * 8 + (i % 8)];
    const uint8_t *y = g.lcode + (size_t)v * g.lstride;
    uint32_t w[4];
#pragma unroll
    for (int e = 0; e < 8; e += 2) {
        float f[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int d = d0 + e + h;
            uint32_t u = (msb >> (7 - ((e + h) & 7))) & 1u;
            if (g.bits > 1) u = (u << (g.bits - 1)) | ex_value(y, g.dim, g.bits - 1, d);
            f[h] = (float)u;
        }
        w[e / 2] = pack_bf16x2(f[0], f[1]);
    }
    *reinterpret_cast<uint4 *>(A + (size_t)v * ix.Dtot + k8) = make_uint4(w[0], w[1], w[2], w[3]);
}

__global__ void k_tc_cluster_of(const int64_t *__restrict__ vec_off, int K, int32_t *__restrict__ cl_of) {
    const int c = blockIdx.x;
    for (int64_t v = vec_off[c] + threadIdx.x; v < vec_off[c + 1]; v += blockDim.x) cl_of[v] = c;
}

// ------------------------------------------------------------ pairs
// One warp per query: candidate offsets of its probes in probe order
// (lp[i][j] = sizes of probes 0..j-1; lp[i][j] for j >= the query's nprobe =
// its candidate count) and the per-cluster pair counts.  qnp: per-query nprobe
// (null: nprobe for every query); probe rows are nprobe long.
__global__ void k_tc_pairs(DevIndexView ix, const uint32_t *__restrict__ probe, int nq, int nprobe,
                           const int *__restrict__ qnp, int *__restrict__ lp, int *__restrict__ qtot,
                           int *__restrict__ bcnt) {
    const int qi = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (qi >= nq) return;
    const int npq = qnp ? qnp[qi] : nprobe;
    int run = 0;
    for (int j0 = 0; j0 < npq; j0 += 32) {
        const int j = j0 + lane;
        int sz = 0;
        if (j < npq) {
            const uint32_t c = probe[(size_t)qi * nprobe + j];
            sz = (int)(ix.vec_off[c + 1] - ix.vec_off[c]);
            atomicAdd(&bcnt[c], 1);
        }
        int x = sz;  // inclusive warp scan
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(kFullMask, x, o);
            if (lane >= o) x += y;
        }
        if (j < npq) lp[(size_t)qi * (nprobe + 1) + j] = run + x - sz;
        run += __shfl_sync(kFullMask, x, 31);
    }
    for (int j = npq + lane; j <= nprobe; j += 32) lp[(size_t)qi * (nprobe + 1) + j] = run;
    if (lane == 0) qtot[qi] = run;
}

// Exclusive prefix sum of n ints into n + 1 int64s (the last is the total);
// one CTA of 1024 threads, each over a contiguous run.
__global__ void __launch_bounds__(1024) k_excl_scan(const int *__restrict__ in, int n, long long *__restrict__ out) {
    __shared__ long long wsum[32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int per = (n + 1023) / 1024, b = min(n, tid * per), e = min(n, b + per);
    long long s = 0;
    for (int i = b; i < e; ++i) s += in[i];
    long long x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(kFullMask, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
        long long t = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(kFullMask, t, o);
            if (lane >= o) t += y;
        }
        wsum[lane] = t;
    }
    __syncthreads();
    long long run = x - s + (w ? wsum[w - 1] : 0);
    for (int i = b; i < e; ++i) {
        out[i] = run;
        run += in[i];
    }
    if (tid == 1023) out[n] = run;
}

__global__ void k_tc_fill(const uint32_t *__restrict__ probe, int npairs, int nprobe, const int *__restrict__ qnp,
                          const long long *__restrict__ boff, int *__restrict__ bfill, int *__restrict__ bucket) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    if (qnp && p % nprobe >= qnp[p / nprobe]) return;  // past this query's nprobe
    const uint32_t c = probe[p];
    const int slot = atomicAdd(&bfill[c], 1);
    bucket[boff[c] + slot] = p;
}

// Each cluster's bucket in ascending pair order (pair = query * nprobe + j):
// rank sort in shared memory, one CTA per cluster.
__global__ void __launch_bounds__(256) k_tc_sort(const int *__restrict__ bcnt, const long long *__restrict__ boff,
                                                 const int *__restrict__ bucket, int *__restrict__ sorted) {
    __shared__ int v[kTcMaxBatch];
    const int c = blockIdx.x, n = bcnt[c];
    if (n == 0) return;
    const int *in = bucket + boff[c];
    int *out = sorted + boff[c];
    for (int e = threadIdx.x; e < n; e += blockDim.x) v[e] = in[e];
    __syncthreads();
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int x = v[e];
        int r = 0;
        for (int k = 0; k < n; ++k) r += v[k] < x;
        out[r] = x;
    }
}

// ------------------------------------------------------------ query operand
// One warp per bucket row b (a (query, probed cluster) pair in cluster order):
// the BF16 residual r = q P - c P of every segment, row-major [b][Dtot], the
// per-segment sum and squared norm of r in FP32 (fixed order: lane-strided
// partials, then a butterfly), and the row's candidate offset.
__global__ void k_tc_gather(DevIndexView ix, const uint32_t *__restrict__ probe, const int *__restrict__ sorted,
                            int P, int nprobe, const float *__restrict__ qrot, const long long *__restrict__ qbase,
                            const int *__restrict__ lp, __nv_bfloat16 *__restrict__ Bq, float2 *__restrict__ pscal,
                            long long *__restrict__ cbase, const long long *__restrict__ ptot) {
    const int b = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (b >= P || (ptot && b >= *ptot)) return;  // ptot: the pairs actually bucketed (P an upper bound)
    const int p = sorted[b], qi = p / nprobe, j = p - qi * nprobe;
    const int c = (int)probe[p];
    if (lane == 0) cbase[b] = qbase[qi] + lp[(size_t)qi * (nprobe + 1) + j];
    const float *qr = qrot + (size_t)qi * ix.Dtot;
    __nv_bfloat16 *out = Bq + (size_t)b * ix.Dtot;
    for (int s = 0; s < ix.S; ++s) {
        const SegDev &g = ix.seg[s];
        const float *cen = g.cent + (size_t)c * g.dim;
        float sum = 0.0f, sq = 0.0f;
        for (int d0 = lane * 8; d0 < g.dim; d0 += 256) {
            const float4 a0 = *reinterpret_cast<const float4 *>(qr + g.qoff + d0);
            const float4 a1 = *reinterpret_cast<const float4 *>(qr + g.qoff + d0 + 4);
            const float4 c0 = *reinterpret_cast<const float4 *>(cen + d0);
            const float4 c1 = *reinterpret_cast<const float4 *>(cen + d0 + 4);
            const float e[8] = {__fsub_rn(a0.x, c0.x), __fsub_rn(a0.y, c0.y), __fsub_rn(a0.z, c0.z),
                                __fsub_rn(a0.w, c0.w), __fsub_rn(a1.x, c1.x), __fsub_rn(a1.y, c1.y),
                                __fsub_rn(a1.z, c1.z), __fsub_rn(a1.w, c1.w)};
#pragma unroll
            for (int h = 0; h < 8; ++h) {
                sum = __fadd_rn(sum, e[h]);
                sq = __fmaf_rn(e[h], e[h], sq);
            }
            *reinterpret_cast<uint4 *>(out + g.qoff + d0) =
                make_uint4(pack_bf16x2(e[0], e[1]), pack_bf16x2(e[2], e[3]), pack_bf16x2(e[4], e[5]),
                           pack_bf16x2(e[6], e[7]));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sum = __fadd_rn(sum, __shfl_xor_sync(kFullMask, sum, o));
            sq = __fadd_rn(sq, __shfl_xor_sync(kFullMask, sq, o));
        }
        if (lane == 0) pscal[(size_t)b * ix.S + s] = make_float2(sum, sq);
    }
}

// ------------------------------------------------------------ contraction
struct TcWork {
    const int2 *tiles;          // (cluster, tile) of every 128-vector tile
    int ntiles;
    const int *bcnt;            // pairs per cluster
    const long long *boff;      // bucket offsets (rows of the query operand)
    const long long *cbase;     // [P] candidate offset of each bucket row
    const float2 *pscal;        // [P][S] residual sum / squared norm per segment
    float *cand;                // approximate distances
    int BN;                     // pairs per chunk (multiple of 16)
    long long cand_cap;         // approximate distances the cand array holds
    int *err;
    // every pipeline wait gives up after wait_ns; skip_it >= 0 (tests of the
    // timeout path only): CTA 0's producer issues no copy for its stage skip_it
    unsigned long long wait_ns;
    int skip_it;
};

// Persistent contraction, one CTA per SM, tiles round-robin.  Roles:
//   warp 0 (one thread)  TMA: per 64-dim stage the 128-row code tile and the
//                        chunk's query rows (16-row boxes), into a 6-stage ring
//   warp 1 (one thread)  tcgen05.mma into one of two TMEM accumulators
//                        (segment s at columns s * BN), commits free the stage /
//                        publish the accumulator; warp 1 also owns TMEM
//   warps 2-5            epilogue: tcgen05.ld of their 32 lanes, the distance
//                        formula, coalesced stores; then hand the accumulator back
// Chunk g uses accumulator g & 1, so the MMAs of chunk g+1 overlap the epilogue
// of chunk g.  Every wait is bounded (mbar_wait): on a timeout the CTA records
// the error, drains its copies and MMAs in flight, frees TMEM and returns.
__global__ void __launch_bounds__(kTcThreads, 1) k_tc_contract(const __grid_constant__ CUtensorMap tmA,
                                                               const __grid_constant__ CUtensorMap tmB,
                                                               DevIndexView ix, TcWork w) {
    extern __shared__ uint8_t tc_smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int S = ix.S, BN = w.BN, kch = ix.Dtot / kTcBK;

    const uint32_t raw = smem_u32(tc_smem);
    const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
    uint8_t *sm = tc_smem + pad;
    const uint32_t sA = raw + pad, sB = sA + kTcStages * kTcStageBytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + 2 * kTcStages * kTcStageBytes);
    const uint32_t b0 = smem_u32(bars);
    auto full = [&](int st) { return b0 + 8u * st; };
    auto empty = [&](int st) { return b0 + 8u * (kTcStages + st); };
    auto accf = [&](int i) { return b0 + 8u * (2 * kTcStages + i); };
    auto acce = [&](int i) { return b0 + 8u * (2 * kTcStages + 2 + i); };
    const uint32_t done = b0 + 8u * (2 * kTcStages + 4);
    int *misc = reinterpret_cast<int *>(bars + 2 * kTcStages + 5);  // [0] TMEM address, [1] abort
    volatile int *abort = misc + 1;

    int ncols = 32;
    while (ncols < 2 * S * BN) ncols <<= 1;
    if (tid == 0) {
        for (int st = 0; st < kTcStages; ++st) {
            mbar_init(full(st), 1);
            mbar_init(empty(st), 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(accf(i), 1);
            mbar_init(acce(i), 4);
        }
        mbar_init(done, 1);
        misc[1] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(misc)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = (uint32_t)misc[0];

    if (warp == 0) {
        // ---- TMA producer
        if (lane == 0) {
            int it = 0;
            bool ok = true;
            for (int ti = blockIdx.x; ti < w.ntiles && ok; ti += gridDim.x) {
                const int2 tile = w.tiles[ti];
                const int cnt = w.bcnt[tile.x];
                const int row0 = (int)(ix.vec_off[tile.x] + (int64_t)tile.y * kTcBM);
                for (int ch = 0; ch * BN < cnt && ok; ++ch) {
                    const int nh = min(BN, cnt - ch * BN), npad = (nh + 15) & ~15;
                    const int brow = (int)(w.boff[tile.x] + (long long)ch * BN);
                    for (int kc = 0; kc < kch; ++kc, ++it) {
                        const int st = it % kTcStages;
                        const uint32_t ph = (uint32_t)(it / kTcStages) & 1u;
                        if (!mbar_wait(empty(st), ph ^ 1u, abort, w.wait_ns)) {
                            ok = false;
                            break;
                        }
                        if (it == w.skip_it && blockIdx.x == 0) continue;  // test hook: this stage never fills
                        mbar_expect_tx(full(st), kTcStageBytes + npad * 128);
                        tma_load_2d(sA + st * kTcStageBytes, &tmA, full(st), kc * kTcBK, row0);
                        for (int bx = 0; bx < npad / 16; ++bx)
                            tma_load_2d(sB + st * kTcStageBytes + bx * 2048, &tmB, full(st), kc * kTcBK, brow + 16 * bx);
                    }
                }
            }
            if (!ok) {
                atomicExch(w.err, 1);
                for (int k = max(0, it - kTcStages); k < it; ++k)  // copies possibly in flight
                    mbar_drain(full(k % kTcStages), (uint32_t)(k / kTcStages) & 1u, w.wait_ns);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        // ---- MMA issuer
        if (lane == 0) {
            int it = 0, g = 0;
            bool ok = true;
            for (int ti = blockIdx.x; ti < w.ntiles && ok; ti += gridDim.x) {
                const int cnt = w.bcnt[w.tiles[ti].x];
                for (int ch = 0; ch * BN < cnt && ok; ++ch, ++g) {
                    const int nh = min(BN, cnt - ch * BN), npad = (nh + 15) & ~15;
                    const uint32_t idesc = idesc_bf16(npad);
                    const int buf = g & 1;
                    if (!mbar_wait(acce(buf), (((uint32_t)g >> 1) & 1u) ^ 1u, abort, w.wait_ns)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t dacc = tmem + (uint32_t)(buf * S * BN);
                    for (int kc = 0; kc < kch; ++kc, ++it) {
                        const int st = it % kTcStages;
                        const uint32_t ph = (uint32_t)(it / kTcStages) & 1u;
                        if (!mbar_wait(full(st), ph, abort, w.wait_ns)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const int k0 = kc * kTcBK;
                        int s = 0;
                        while (s + 1 < S && k0 >= ix.seg[s + 1].qoff) ++s;
                        const bool first = k0 == ix.seg[s].qoff;
                        const uint64_t da = sw128_desc(sA + st * kTcStageBytes), db = sw128_desc(sB + st * kTcStageBytes);
#pragma unroll
                        for (int kk = 0; kk < kTcBK / 16; ++kk)  // 16 BF16 = 32 bytes per instruction
                            mma_bf16(dacc + (uint32_t)(s * BN), da + 2 * kk, db + 2 * kk, idesc,
                                     (first && kk == 0) ? 0u : 1u);
                        mma_commit(empty(st));
                    }
                    if (ok) mma_commit(accf(buf));
                }
            }
            if (!ok) atomicExch(w.err, 1);
            mma_commit(done);  // every MMA issued has finished once `done` completes
            mbar_drain(done, 0, w.wait_ns);
        }
        __syncwarp();
    } else {
        // ---- epilogue: warps 2-5, TMEM lanes (warp % 4) * 32 + lane
        const int qt = warp & 3, r = qt * 32 + lane;
        int g = 0;
        bool ok = true;
        for (int ti = blockIdx.x; ti < w.ntiles && ok; ti += gridDim.x) {
            const int2 tile = w.tiles[ti];
            const int c = tile.x, cnt = w.bcnt[c];
            if (cnt == 0) continue;
            const int64_t v0 = ix.vec_off[c];
            const int nc = (int)(ix.vec_off[c + 1] - v0);
            const int rl = tile.y * kTcBM + r;
            const bool vrow = rl < nc;
            const int64_t gv = v0 + rl, gb = ix.blk_off[c] + rl / 32;
            const int ln = rl & 31;
            for (int ch = 0; ch * BN < cnt; ++ch, ++g) {
                const int nh = min(BN, cnt - ch * BN), npad = (nh + 15) & ~15;
                const int buf = g & 1;
                if (ok && !mbar_wait(accf(buf), ((uint32_t)g >> 1) & 1u, abort, w.wait_ns)) ok = false;
                tc_fence_after();
                if (!__all_sync(kFullMask, ok)) {
                    ok = false;
                    break;
                }
                const long long rb = w.boff[c] + (long long)ch * BN;
                for (int n0 = 0; n0 < npad; n0 += 16) {
                    float d[16];
#pragma unroll
                    for (int i = 0; i < 16; ++i) d[i] = 0.0f;
                    for (int s = 0; s < S; ++s) {
                        float v[16];
                        tmem_ld16(tmem + ((uint32_t)(qt * 32) << 16) + (uint32_t)(buf * S * BN + s * BN + n0), v);
                        const SegDev &sg = ix.seg[s];
                        const float on = vrow ? sg.onorm[gb * 32 + ln] : 0.0f;
                        const float o2 = __fmul_rn(on, on), rs = vrow ? sg.exfac[gv].x : 0.0f;
                        const float dl = 2.0f / (float)(1 << sg.bits), cst = __fsub_rn(__fmul_rn(dl, 0.5f), 1.0f);
#pragma unroll
                        for (int i = 0; i < 16; ++i) {
                            const int n = n0 + i;
                            const float2 ps = n < nh ? w.pscal[(rb + n) * S + s] : make_float2(0.0f, 0.0f);
                            const float ip = __fmaf_rn(dl, v[i], __fmul_rn(cst, ps.x));
                            d[i] = __fadd_rn(d[i], __fsub_rn(__fadd_rn(o2, ps.y), __fmul_rn(2.0f, __fmul_rn(rs, ip))));
                        }
                    }
                    if (vrow) {
#pragma unroll
                        for (int i = 0; i < 16; ++i)
                            if (n0 + i < nh) {
                                const long long at = w.cbase[rb + n0 + i] + rl;
                                if (at < w.cand_cap) w.cand[at] = d[i];
                            }
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(acce(buf));
            }
        }
        if (!ok && lane == 0) atomicExch(w.err, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
    }
}

constexpr size_t tc_contract_smem() { return 1024 + 2 * (size_t)kTcStages * kTcStageBytes + 8 * (2 * kTcStages + 5) + 16; }

// ------------------------------------------------------------ shortlist
__device__ __forceinline__ uint32_t dkey(float f) {
    if (f != f) return 0xffffffffu;
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Block-wide exclusive scan of a 0/1 flag (256 threads); returns the prefix
// and the block total in *tot.
__device__ __forceinline__ int block_prefix(int f, int *wtot, int *tot) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned b = __ballot_sync(kFullMask, f);
    if (lane == 0) wtot[w] = __popc(b);
    __syncthreads();
    int base = 0, all = 0;
    for (int i = 0; i < 8; ++i) {
        base += i < w ? wtot[i] : 0;
        all += wtot[i];
    }
    __syncthreads();
    *tot = all;
    return base + __popc(b & ((1u << lane) - 1u));
}

// The L smallest keys of key(e), e in [0, M) (ties: smaller e first), written
// in ascending e as (pos(e), value(e)).  256 threads; radix select, 8 bits per pass.
template <class Key, class Emit>
__device__ void select_smallest(int M, int L, Key key, Emit emit) {
    __shared__ int hist[256];
    __shared__ int wtot[8];
    __shared__ uint32_t s_prefix;
    __shared__ int s_need;
    const int tid = threadIdx.x;
    uint32_t prefix = 0, mask = 0;
    int need = L;
    for (int shift = 24; shift >= 0; shift -= 8) {
        hist[tid] = 0;
        __syncthreads();
        for (int e = tid; e < M; e += 256) {
            const uint32_t k = key(e);
            if ((k & mask) == prefix) atomicAdd(&hist[(k >> shift) & 255], 1);
        }
        __syncthreads();
        if (tid == 0) {
            int acc = 0, b = 0;
            while (acc + hist[b] < need) acc += hist[b++];
            s_prefix = prefix | ((uint32_t)b << shift);
            s_need = need - acc;
        }
        __syncthreads();
        prefix = s_prefix;
        need = s_need;
        mask |= 255u << shift;
        __syncthreads();
    }
    int taken = 0, eq_seen = 0;
    for (int e0 = 0; e0 < M; e0 += 256) {
        const int e = e0 + tid;
        const uint32_t k = e < M ? key(e) : 0xffffffffu;
        const int lt = e < M && k < prefix, eq = e < M && k == prefix;
        int eq_tot;
        const int eq_rank = eq_seen + block_prefix(eq, wtot, &eq_tot);
        const int f = lt || (eq && eq_rank < need);
        int f_tot;
        const int slot = taken + block_prefix(f, wtot, &f_tot);
        if (f) emit(slot, e);
        taken += f_tot;
        eq_seen += eq_tot;
    }
}

constexpr int kTcSelChunk = 4096;  // candidates per first-phase CTA

// Phase 1: the L smallest of each 4,096-candidate chunk of a query (chunks of
// all queries concatenated: qchunk = exclusive prefix of chunks per query),
// padded to L entries with (INT_MAX, NaN) so each query's survivors are a
// dense array in candidate order.
__global__ void __launch_bounds__(256) k_tc_select1(const float *__restrict__ cand, const long long *__restrict__ qbase,
                                                    const int *__restrict__ qtot, const long long *__restrict__ qchunk,
                                                    int nq, int L, int *__restrict__ spos, float *__restrict__ sval) {
    __shared__ float xs[kTcSelChunk];
    const long long k = blockIdx.x;
    if (k >= qchunk[nq]) return;  // a grid sized by a capacity (graph launches)
    int lo = 0, hi = nq - 1;  // query owning chunk k: last with qchunk <= k
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (qchunk[mid] <= k) lo = mid;
        else hi = mid - 1;
    }
    const int qi = lo;
    const int e0 = (int)(k - qchunk[qi]) * kTcSelChunk, m = min(kTcSelChunk, qtot[qi] - e0);
    const float *x = cand + qbase[qi] + e0;
    for (int e = threadIdx.x; e < m; e += 256) xs[e] = x[e];
    __syncthreads();
    int *po = spos + k * L;
    float *vo = sval + k * L;
    if (m <= L) {
        for (int e = threadIdx.x; e < L; e += 256) {
            po[e] = e < m ? e0 + e : INT_MAX;
            vo[e] = e < m ? xs[e] : __int_as_float(0x7fffffff);
        }
        return;
    }
    select_smallest(m, L, [&](int e) { return dkey(xs[e]); },
                    [&](int slot, int e) {
                        po[slot] = e0 + e;
                        vo[slot] = xs[e];
                    });
}

// Phase 2: per query, the L smallest of its survivors (ties: earlier position),
// in candidate order.
__global__ void __launch_bounds__(256) k_tc_select2(const long long *__restrict__ qchunk, const int *__restrict__ qtot,
                                                    int L, const int *__restrict__ spos, const float *__restrict__ sval,
                                                    int *__restrict__ sl_pos, float *__restrict__ sl_apx,
                                                    int *__restrict__ sl_cnt) {
    const int qi = blockIdx.x;
    const int M = qtot[qi];
    const long long c0 = qchunk[qi];
    const int n = (int)(qchunk[qi + 1] - c0) * L;
    const int *pi = spos + c0 * L;
    const float *vi = sval + c0 * L;
    int *po = sl_pos + (size_t)qi * L;
    float *ao = sl_apx + (size_t)qi * L;
    const int take = min(L, M);
    if (threadIdx.x == 0) sl_cnt[qi] = take;
    if (M <= L) {  // one chunk holding every candidate, in order
        for (int e = threadIdx.x; e < M; e += 256) {
            po[e] = pi[e];
            ao[e] = vi[e];
        }
        return;
    }
    // padding (INT_MAX, NaN) has the largest key and comes last on ties
    select_smallest(n, L, [&](int e) { return dkey(vi[e]); },
                    [&](int slot, int e) {
                        po[slot] = pi[e];
                        ao[slot] = vi[e];
                    });
}

// Calls without a host round trip (graph launches): when the batch needs more
// approximate distances than `cap` or more selection chunks than `chunk_cap`,
// record it (bit 2 of the error word) and empty every bucket and candidate
// count, so that no later kernel reads or writes past the arrays.
__global__ void k_tc_guard(const long long *__restrict__ qbase, const long long *__restrict__ qchunk, int nq, int K,
                           long long cap, long long chunk_cap, int *__restrict__ bcnt, int *__restrict__ qtot,
                           int *__restrict__ err) {
    if (qbase[nq] <= cap && qchunk[nq] <= chunk_cap) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    if (i == 0) atomicOr(err, 2);
    for (int c = i; c < K; c += stride) bcnt[c] = 0;
    for (int q = i; q < nq; q += stride) qtot[q] = 0;
}

__global__ void k_tc_chunks(const int *__restrict__ qtot, int nq, int *__restrict__ nch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nq) nch[i] = (qtot[i] + kTcSelChunk - 1) / kTcSelChunk;
}

}  // namespace

// ------------------------------------------------------------ host
namespace {

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    if (!fn) throw Error{SAQG_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver"};
    return fn;
}

// The BF16 code matrix and the tile list of an index, built on first use.
void ensure_tc_state(const Index &I, cudaStream_t st) {
    std::lock_guard<std::mutex> lk(I.init_mu);
    if (I.tc_codes) return;
    const DevIndexView &ix = I.view;
    const size_t bytes = 2 * (size_t)I.N * ix.Dtot;
    void *A = nullptr, *cl = nullptr, *tiles = nullptr;
    std::vector<int2> ht;
    for (int64_t c = 0; c < I.K; ++c)
        for (int64_t t = 0; t * kTcBM < I.sizes[c]; ++t) ht.push_back(make_int2((int)c, (int)t));
    SAQG_CUDA_TRY(cudaMalloc(&A, std::max<size_t>(bytes, 16)));
    try {
        SAQG_CUDA_TRY(cudaMalloc(&cl, 4 * std::max<size_t>(1, (size_t)I.N)));
        SAQG_CUDA_TRY(cudaMalloc(&tiles, sizeof(int2) * std::max<size_t>(1, ht.size())));
        if (!ht.empty())
            SAQG_CUDA_TRY(cudaMemcpyAsync(tiles, ht.data(), sizeof(int2) * ht.size(), cudaMemcpyHostToDevice, st));
        if (I.N > 0) {
            k_tc_cluster_of<<<(unsigned)I.K, 256, 0, st>>>(ix.vec_off, (int)I.K, static_cast<int32_t *>(cl));
            const int64_t work = I.N * (ix.Dtot / 8);
            k_tc_codes<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(ix, static_cast<const int32_t *>(cl), I.N,
                                                                      static_cast<__nv_bfloat16 *>(A));
            const cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) throw Error{SAQG_ERR_CUDA, std::string("k_tc_codes launch failed: ") + cudaGetErrorString(e)};
            count_launch(2);
        }
        SAQG_CUDA_TRY(cudaStreamSynchronize(st));
    } catch (...) {
        cudaFree(A);
        if (cl) cudaFree(cl);
        if (tiles) cudaFree(tiles);
        throw;
    }
    cudaFree(cl);
    I.tc_codes = A;
    I.tc_tiles = tiles;
    I.tc_ntiles = (int64_t)ht.size();
}

void launch_check(const char *what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error{SAQG_ERR_CUDA, std::string(what) + " launch failed: " + cudaGetErrorString(e)};
}

size_t a16(size_t x) { return (x + 15) & ~size_t(15); }

int sm_count() {
    static int n = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
    });
    return n;
}

CUtensorMap bf16_rows_map(void *base, int64_t cols, int64_t rows, int box_rows) {
    CUtensorMap m;
    const cuuint64_t gdim[2] = {(cuuint64_t)cols, (cuuint64_t)std::max<int64_t>(rows, 1)};
    const cuuint64_t gstride[1] = {(cuuint64_t)cols * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kTcBK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = tensor_map_encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, gdim, gstride, box, estr,
                                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error{SAQG_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r)};
    return m;
}

}  // namespace

namespace {

// Pairs per MMA chunk: the tuned value when given (a multiple of 16), at most
// what two accumulators of S segments fit in TMEM.
int tc_bn(const DevIndexView &ix, int tuned) {
    const int cap = std::min(kTcMaxN, (kTcCols / ix.S) / 16 * 16);
    if (tuned >= 16) return std::min(cap, tuned / 16 * 16);
    return cap;
}

// Scratch layout of one call: arena 1 by the call's shape, arena 2 by its
// candidates (the exact count, or a capacity for calls without a host round trip).
size_t tc_arena1_bytes(const Index &I, int64_t nq, int64_t topk, int64_t nprobe, int64_t L) {
    const DevIndexView &ix = I.view;
    const int64_t P = nq * nprobe;
    size_t need = 0;
    auto add = [&](size_t b) { need += a16(b); };
    add(4 * (size_t)nq * I.D);                  // queries
    add(4 * (size_t)nq * I.K);                  // centroid distances
    add(tc_probe_work_bytes(I, nq));            // selection work
    add(4 * (size_t)P);                         // probes
    add(4 * (size_t)nq * ix.Dtot);              // rotated queries
    add(4 * (size_t)nq * ix.S);                 // prune bounds
    add(2 * (size_t)nq * I.D);                  // BF16 queries (probe GEMM)
    add((size_t)nq);                            // full-path flags
    add(4 * (size_t)nq);                        // full-path list
    add(64);                                    // flags
    add(4 * (size_t)nq * (nprobe + 1));         // lp
    add(4 * (size_t)nq * 2);                    // qtot, chunks per query
    add(8 * (size_t)(nq + 1) * 2);              // qbase, qchunk
    add(4 * (size_t)I.K * 2);                   // bcnt, bfill
    add(8 * (size_t)(I.K + 1));                 // boff
    add(4 * (size_t)P * 2);                     // bucket, sorted
    add(4 * (size_t)nq * L * 5);                // sl_pos, sl_apx, sl_dist, groups, group probes
    add(4 * (size_t)nq * 2);                    // sl_cnt, group counts
    add(4 * (size_t)nq * topk * 3);             // outputs (host io)
    add(16);                                    // error word
    add(4 * (size_t)nq * 2);                    // per-query nprobe / k
    return need + 256;
}

size_t tc_arena2_bytes(const DevIndexView &ix, int64_t total, int64_t pairs, int64_t nchunks, int64_t L) {
    return a16(4 * (size_t)std::max<int64_t>(total, 1)) + a16(2 * (size_t)pairs * ix.Dtot) +
           a16(8 * (size_t)pairs * ix.S) + a16(8 * (size_t)pairs) +
           a16(8 * (size_t)std::max<int64_t>(nchunks, 1) * L) + 256;
}

}  // namespace

void presize_tc_ctx(const Index &I, SearchCtx &C, int64_t nq, int64_t topk, int64_t nprobe, int64_t L,
                    int64_t cand_cap) {
    std::lock_guard<std::mutex> lock(C.mu);
    C.scratch_get(tc_arena1_bytes(I, nq, topk, nprobe, L));
    C.split_scratch_get(tc_arena2_bytes(I.view, cand_cap, nq * nprobe, cand_cap / kTcSelChunk + nq, L));
}

void run_search_tc(const Index &I, const float *q, int64_t nq, int64_t topk, int64_t nprobe, int64_t L, float m,
                   uint32_t *ids, float *dists, float *approx, int mem, cudaStream_t st, saqg_tc_stats *stats,
                   const int *np_host, const int *k_host, const TcOpts *opts) {
    const DevIndexView &ix = I.view;
    const TcOpts none;
    const TcOpts &o = opts ? *opts : none;
    const bool dev_shape = !np_host && !k_host && (o.np_dev || o.k_dev);
    // per-query nprobe / k (host arrays): the scalars become their maxima
    int64_t pairs = nq * nprobe;
    if (np_host || k_host) {
        int64_t npm = 0, km = 0;
        pairs = 0;
        for (int64_t i = 0; i < nq; ++i) {
            const int a = np_host ? np_host[i] : (int)nprobe, b = k_host ? k_host[i] : (int)topk;
            SAQG_REQUIRE(a >= 1 && a <= I.K, "every nprobe must be in [1, number of clusters]");
            SAQG_REQUIRE(b >= 1 && b <= kTcMaxShort, "every topk must be in [1, 1024]");
            npm = std::max<int64_t>(npm, a);
            km = std::max<int64_t>(km, b);
            pairs += a;
        }
        if (np_host) nprobe = npm;
        if (k_host) topk = km;
    }
    SAQG_REQUIRE(nq >= 0 && nq <= kTcMaxBatch, "the tensor-core search takes at most 8192 queries per call");
    SAQG_REQUIRE(topk >= 1 && topk <= kTcMaxShort, "topk must be in [1, 1024]");
    SAQG_REQUIRE(L >= topk && L <= kTcMaxShort, "shortlist must be in [topk, 1024]");
    SAQG_REQUIRE(nprobe >= 1 && nprobe <= I.K, "nprobe must be in [1, number of clusters]");
    SAQG_REQUIRE(o.cand_cap >= 0 && o.cand_cap < ((int64_t)1 << 40), "candidate capacity out of range");
    for (int s = 0; s < ix.S; ++s)
        SAQG_REQUIRE(ix.seg[s].bits >= 1 && ix.seg[s].dim % kTcBK == 0,
                     "the tensor-core search needs every segment coded (bits >= 1) and 64-dim aligned");
    SAQG_REQUIRE(I.N < (int64_t)1 << 31 && nq * nprobe < (int64_t)1 << 31, "index or batch too large");
    if (nq == 0) return;
    TcTune tune;
    if (o.tune) {
        tune = *o.tune;
    } else {
        std::lock_guard<std::mutex> lk(I.tune_mu);
        const auto it = I.tc_tunes.find(TuneKey{1, tune_bucket(nq), topk, nprobe});
        if (it != I.tc_tunes.end()) tune = it->second;
    }
    const int BN = tc_bn(ix, tune.bn);
    SAQG_REQUIRE(BN >= 16, "too many segments for the tensor-core search");
    ensure_tc_state(I, st);

    std::unique_ptr<CtxLease> lease;
    SearchCtx *ctxp = o.ctx;
    if (!ctxp) {
        lease = std::make_unique<CtxLease>(I, st);  // locked; ordered after its previous call
        ctxp = lease->c;
    }
    SearchCtx &C = *ctxp;
    std::unique_lock<std::mutex> lock(C.mu, std::defer_lock);
    if (!lease) lock.lock();  // the caller's own context (graph)
    const bool host = mem == SAQG_MEM_HOST;
    const bool capped = o.cand_cap > 0;  // no host round trip
    const int64_t P = nq * nprobe;  // probe slots (rows of nprobe); `pairs` of them are used
    char *base = static_cast<char *>(C.scratch_get(tc_arena1_bytes(I, nq, topk, nprobe, L)));
    size_t off = 0;
    auto take = [&](size_t b) {
        char *p = base + off;
        off += a16(b);
        return p;
    };
    float *dq = reinterpret_cast<float *>(take(4 * (size_t)nq * I.D));
    float *dist = reinterpret_cast<float *>(take(4 * (size_t)nq * I.K));
    void *work = take(tc_probe_work_bytes(I, nq));
    uint32_t *probe = reinterpret_cast<uint32_t *>(take(4 * (size_t)P));
    float *qrot = reinterpret_cast<float *>(take(4 * (size_t)nq * ix.Dtot));
    float *prune = reinterpret_cast<float *>(take(4 * (size_t)nq * ix.S));
    void *qbf = take(2 * (size_t)nq * I.D);
    uint8_t *full = reinterpret_cast<uint8_t *>(take((size_t)nq));
    int *fb = reinterpret_cast<int *>(take(4 * (size_t)nq));
    int *flags = reinterpret_cast<int *>(take(64));
    int *lp = reinterpret_cast<int *>(take(4 * (size_t)nq * (nprobe + 1)));
    int *qtot = reinterpret_cast<int *>(take(4 * (size_t)nq * 2));
    int *nchk = qtot + nq;
    long long *qbase = reinterpret_cast<long long *>(take(8 * (size_t)(nq + 1) * 2));
    long long *qchunk = qbase + nq + 1;
    int *bcnt = reinterpret_cast<int *>(take(4 * (size_t)I.K * 2));
    int *bfill = bcnt + I.K;
    long long *boff = reinterpret_cast<long long *>(take(8 * (size_t)(I.K + 1)));
    int *bucket = reinterpret_cast<int *>(take(4 * (size_t)P * 2));
    int *sorted = bucket + P;
    int *sl_pos = reinterpret_cast<int *>(take(4 * (size_t)nq * L * 5));
    float *sl_apx = reinterpret_cast<float *>(sl_pos + nq * L);
    float *sl_dist = sl_apx + nq * L;
    int *grp = reinterpret_cast<int *>(sl_dist + nq * L);
    int *gj = grp + nq * L;
    int *sl_cnt = reinterpret_cast<int *>(take(4 * (size_t)nq * 2));
    int *ng = sl_cnt + nq;
    uint32_t *oid = reinterpret_cast<uint32_t *>(take(4 * (size_t)nq * topk * 3));
    float *od = reinterpret_cast<float *>(oid + nq * topk);
    float *oa = od + nq * topk;
    int *err = reinterpret_cast<int *>(take(16));
    if (o.err_word) *o.err_word = err;
    int *qnp = nullptr, *qk = nullptr;
    {
        int *pk = reinterpret_cast<int *>(take(4 * (size_t)nq * 2));
        if (np_host) {
            qnp = pk;
            SAQG_CUDA_TRY(cudaMemcpyAsync(qnp, np_host, 4 * (size_t)nq, cudaMemcpyHostToDevice, st));
        }
        if (k_host) {
            qk = pk + nq;
            SAQG_CUDA_TRY(cudaMemcpyAsync(qk, k_host, 4 * (size_t)nq, cudaMemcpyHostToDevice, st));
        }
        if (dev_shape) {
            qnp = o.np_dev ? pk : nullptr;
            qk = o.k_dev ? pk + nq : nullptr;
            clamp_shape(o.np_dev, o.k_dev, nq, (int)nprobe, (int)topk, qnp, qk, st);
        }
    }

    cudaEvent_t ev[6] = {};
    struct EvGuard {
        cudaEvent_t *e;
        ~EvGuard() {
            for (int i = 0; i < 6; ++i)
                if (e[i]) cudaEventDestroy(e[i]);
        }
    } evg{ev};
    if (stats)
        for (auto &e : ev) SAQG_CUDA_TRY(cudaEventCreate(&e));
    auto mark = [&](int i) {
        if (stats) SAQG_CUDA_TRY(cudaEventRecord(ev[i], st));
    };

    const float *qin = q;
    if (host) {
        SAQG_CUDA_TRY(cudaMemcpyAsync(dq, q, 4 * (size_t)nq * I.D, cudaMemcpyHostToDevice, st));
        qin = dq;
    }
    mark(0);
    tc_rank_rotate(I, C, qin, nq, nprobe, qnp, m, dist, work, probe, qrot, prune, full, fb, flags, qbf, st);
    mark(1);
    // pairs: candidate offsets per query, buckets per cluster, selection chunks
    SAQG_CUDA_TRY(cudaMemsetAsync(bcnt, 0, 8 * (size_t)I.K, st));
    SAQG_CUDA_TRY(cudaMemsetAsync(err, 0, 16, st));
    k_tc_pairs<<<(unsigned)((nq + 7) / 8), 256, 0, st>>>(ix, probe, (int)nq, (int)nprobe, qnp, lp, qtot, bcnt);
    launch_check("k_tc_pairs");
    k_excl_scan<<<1, 1024, 0, st>>>(qtot, (int)nq, qbase);
    launch_check("k_excl_scan");
    k_tc_chunks<<<(unsigned)((nq + 255) / 256), 256, 0, st>>>(qtot, (int)nq, nchk);
    launch_check("k_tc_chunks");
    k_excl_scan<<<1, 1024, 0, st>>>(nchk, (int)nq, qchunk);
    launch_check("k_excl_scan");
    k_excl_scan<<<1, 1024, 0, st>>>(bcnt, (int)I.K, boff);
    launch_check("k_excl_scan");
    k_tc_fill<<<(unsigned)((P + 255) / 256), 256, 0, st>>>(probe, (int)P, (int)nprobe, qnp, boff, bfill, bucket);
    launch_check("k_tc_fill");
    k_tc_sort<<<(unsigned)I.K, 256, 0, st>>>(bcnt, boff, bucket, sorted);
    launch_check("k_tc_sort");
    long long total = 0, nchunks = 0;
    if (capped) {  // sized by the capacity; a batch beyond it is emptied and reported
        total = o.cand_cap;
        nchunks = o.cand_cap / kTcSelChunk + nq;
        pairs = P;
        k_tc_guard<<<64, 256, 0, st>>>(qbase, qchunk, (int)nq, (int)I.K, total, nchunks, bcnt, qtot, err);
        launch_check("k_tc_guard");
    } else {
        long long totals[2] = {0, 0};
        SAQG_CUDA_TRY(cudaMemcpyAsync(&totals[0], qbase + nq, 8, cudaMemcpyDeviceToHost, st));
        SAQG_CUDA_TRY(cudaMemcpyAsync(&totals[1], qchunk + nq, 8, cudaMemcpyDeviceToHost, st));
        SAQG_CUDA_TRY(cudaStreamSynchronize(st));
        total = totals[0];
        nchunks = totals[1];
        if (dev_shape) pairs = P;
        if (o.candidates) *o.candidates = total;
    }
    // arena 2: sized by the candidates
    char *base2 = static_cast<char *>(C.split_scratch_get(tc_arena2_bytes(ix, total, pairs, nchunks, L)));
    size_t off2 = 0;
    auto take2 = [&](size_t b) {
        char *p = base2 + off2;
        off2 += a16(b);
        return p;
    };
    float *cand = reinterpret_cast<float *>(take2(4 * (size_t)std::max<long long>(total, 1)));
    __nv_bfloat16 *Bq = reinterpret_cast<__nv_bfloat16 *>(take2(2 * (size_t)pairs * ix.Dtot));
    float2 *pscal = reinterpret_cast<float2 *>(take2(8 * (size_t)pairs * ix.S));
    long long *cbase = reinterpret_cast<long long *>(take2(8 * (size_t)pairs));
    int *spos = reinterpret_cast<int *>(take2(8 * (size_t)std::max<long long>(nchunks, 1) * L));
    float *sval = reinterpret_cast<float *>(spos + std::max<long long>(nchunks, 1) * L);
    k_tc_gather<<<(unsigned)((pairs * 32 + 255) / 256), 256, 0, st>>>(ix, probe, sorted, (int)pairs, (int)nprobe, qrot,
                                                                     qbase, lp, Bq, pscal, cbase,
                                                                     pairs == P && (capped || dev_shape) ? boff + I.K
                                                                                                          : nullptr);
    launch_check("k_tc_gather");
    mark(2);
    // contraction: persistent, one CTA per SM
    const CUtensorMap tmA = bf16_rows_map(I.tc_codes, ix.Dtot, I.N, kTcBM);
    const CUtensorMap tmB = bf16_rows_map(Bq, ix.Dtot, pairs, 16);
    TcWork wk;
    wk.tiles = static_cast<const int2 *>(I.tc_tiles);
    wk.ntiles = (int)I.tc_ntiles;
    wk.bcnt = bcnt;
    wk.boff = boff;
    wk.cbase = cbase;
    wk.pscal = pscal;
    wk.cand = cand;
    wk.BN = BN;
    wk.cand_cap = std::max<long long>(total, 1);
    wk.err = err;
    wk.wait_ns = 1000000000ull;
    wk.skip_it = -1;
    // test hooks of the timeout path (tests/test_tc_search.py): a shorter wait
    // limit and one stage of CTA 0 that never fills
    if (const char *e = std::getenv("SAQG_TEST_TC_WAIT_MS")) wk.wait_ns = 1000000ull * (unsigned long long)std::max(1, std::atoi(e));
    if (const char *e = std::getenv("SAQG_TEST_TC_SKIP_STAGE")) wk.skip_it = std::max(0, std::atoi(e));
    const size_t smem = tc_contract_smem();
    SAQG_CUDA_TRY(cudaFuncSetAttribute(k_tc_contract, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (I.tc_ntiles > 0) {
        const unsigned grid = (unsigned)std::min<int64_t>(I.tc_ntiles, sm_count());
        k_tc_contract<<<grid, kTcThreads, smem, st>>>(tmA, tmB, ix, wk);
        launch_check("k_tc_contract");
    }
    mark(3);
    k_tc_select1<<<(unsigned)std::max<long long>(nchunks, 1), 256, 0, st>>>(cand, qbase, qtot, qchunk, (int)nq, (int)L,
                                                                            spos, sval);
    launch_check("k_tc_select1");
    k_tc_select2<<<(unsigned)nq, 256, 0, st>>>(qchunk, qtot, (int)L, spos, sval, sl_pos, sl_apx, sl_cnt);
    launch_check("k_tc_select2");
    mark(4);
    tc_rerank(I, probe, nq, nprobe, qrot, prune, lp, sl_pos, sl_apx, sl_cnt, (int)L, topk, qk, grp, gj, ng, sl_dist,
              host ? oid : ids, host ? od : dists, host ? oa : approx, st);
    mark(5);
    count_launch(capped ? 12 : 11);
    if (host) {
        SAQG_CUDA_TRY(cudaMemcpyAsync(ids, oid, 4 * (size_t)nq * topk, cudaMemcpyDeviceToHost, st));
        if (dists) SAQG_CUDA_TRY(cudaMemcpyAsync(dists, od, 4 * (size_t)nq * topk, cudaMemcpyDeviceToHost, st));
        if (approx) SAQG_CUDA_TRY(cudaMemcpyAsync(approx, oa, 4 * (size_t)nq * topk, cudaMemcpyDeviceToHost, st));
    }
    if (capped && !host && !stats) return;  // the caller reads the error word (graph status)
    int herr = 0;
    SAQG_CUDA_TRY(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
    SAQG_CUDA_TRY(cudaStreamSynchronize(st));
    if (herr & 1) throw Error{SAQG_ERR_INTERNAL, "tensor-core contraction: a pipeline wait timed out"};
    if (herr & 2) throw Error{SAQG_ERR_NOMEM, "tensor-core search: the batch needs more approximate distances than "
                                               "the candidate capacity"};
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        float t[5] = {0, 0, 0, 0, 0};
        for (int i = 0; i < 5; ++i) SAQG_CUDA_TRY(cudaEventElapsedTime(&t[i], ev[i], ev[i + 1]));
        stats->ms_probe = t[0];
        stats->ms_pairs = t[1];
        stats->ms_contract = t[2];
        stats->ms_select = t[3];
        stats->ms_rerank = t[4];
        std::vector<int> hc((size_t)I.K);
        SAQG_CUDA_TRY(cudaMemcpy(hc.data(), bcnt, 4 * (size_t)I.K, cudaMemcpyDeviceToHost));
        int64_t flops = 0, bytes = 0, tiles = 0, padded = 0, npairs = 0;
        for (int64_t c = 0; c < I.K; ++c) {
            if (!hc[c]) continue;
            const int64_t nt = (I.sizes[c] + kTcBM - 1) / kTcBM;
            flops += 2 * (int64_t)ix.Dtot * hc[c] * I.sizes[c];
            bytes += 2 * (int64_t)ix.Dtot * I.sizes[c];
            tiles += nt;
            npairs += hc[c];
            const int64_t nch = (hc[c] + BN - 1) / BN, npad = (nch - 1) * BN + (((hc[c] - (nch - 1) * BN) + 15) & ~15);
            padded += 2 * (int64_t)ix.Dtot * kTcBM * nt * npad;
        }
        long long tot = total;
        if (capped) SAQG_CUDA_TRY(cudaMemcpy(&tot, qbase + nq, 8, cudaMemcpyDeviceToHost));
        stats->pairs = npairs;
        stats->candidates = tot;
        stats->tiles = tiles;
        stats->flops = flops;
        stats->mma_flops = padded;
        stats->code_bytes = bytes;
    }
}

}  // namespace saqg
