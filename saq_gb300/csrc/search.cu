// Search hot path: IVF::search / IVF::estimate (index/ivf.hpp:275-362) on the GPU.
//
// Pipeline for a batch of nq independent queries (nq = 1 is the plain
// single-query drop-in):
//   k_probe_dist   L2 from every query to every centroid, in Eigen's order
//                  (FlatInitializer::centroids_distances, initializer.hpp:52-76)
//   k_probe_select the nprobe nearest in std::partial_sort order: radix select
//                  + sort; on any tie the exact libstdc++ heap algorithm runs
//   k_qprep        per segment: zero-padded query slice, prune bound
//                  sqrt(sum var*q^2)*m and the rotated query q_s*P_s in Eigen's
//                  GEMV order (saq_estimator.hpp:28-48, caq_estimator.hpp:56-68)
//   k_scan         one CTA per query walks its probes in order.  Per cluster:
//                  LUTs (Lut::prepare, lut.hpp:60-87); per tile of blocks
//                  (one warp = one 32-vector block): FastScan sums and fast /
//                  variance estimates, the block's pruning stages, accurate
//                  distances of every lane that can pass under the tile-start
//                  distk (distk only shrinks, so this is a superset), then one
//                  thread replays SAQSearcher::searchCluster / scanCluster
//                  (saq_searcher.hpp:68-214) and the ResultPool inserts
//                  (utils/pool.hpp:17-30) exactly in the reference's order.
#include <cfloat>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <tuple>

#include "device_common.cuh"
#include "saqg_internal.h"

namespace saqg {

namespace {

constexpr int kScanWarps = 8;
constexpr int kScanThreads = kScanWarps * 32;
constexpr int kBlocksPerWarp = 2;
constexpr int kTileB = kScanWarps * kBlocksPerWarp;  // blocks per tile
constexpr int kMaxTopK = 4096;
constexpr int kScanMinCtas = 4;  // resident scan CTAs per SM the register budget is sized for

struct SegScal {
    float delta, vl, sum_vl, sum_q, q_l2sqr, q_l2norm, c1, c2, vfac;
    float rdelta;  // RN(1 / delta): the LUT quantizer's fast path
};

// A u16 LUT entry (uint16_t)(int)(x / d), x >= 0, with the division rounded to
// nearest, mostly without dividing: y = RN(x * r), r = RN(1 / d), lies within
// 3.02 * 2^-24 * y of RN(x / d), so when no integer lies within 2^-21 * y of y
// both truncate to the same integer.  Otherwise (and for NaN / inf) `ok` is
// false and the caller divides.  The floors come from adding 2^23 rounded
// down (2^23 + floor(v) for 0 <= v < 2^23, the integer in the low mantissa
// bits), so the check and the result take FP32 adds, not conversions.
__device__ __forceinline__ uint32_t lut_quant_fast(float x, float r, bool &ok) {
    const float y = __fmul_rn(x, r);
    const float e = __fmul_rn(y, 4.76837158203125e-07f);  // 2^-21
    const float lo = __fadd_rd(__fsub_rn(y, e), 8388608.0f), hi = __fadd_rd(__fadd_rn(y, e), 8388608.0f);
    ok = lo == hi && y < 4194304.0f;  // y < 2^22 keeps both sums in the binade of 2^23
    return __float_as_uint(lo) & 0xffffu;  // (uint16_t)(int)y: y >= 0, trunc = floor
}

__device__ __forceinline__ uint32_t fkey(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float key_to_float(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Per-query nprobe and k of a batch (null arrays: every query uses the
// maxima).  Probe rows are np_max long and result rows k_max long.
struct QueryShape {
    const int *np = nullptr, *k = nullptr;
    int np_max = 0, k_max = 0;
    __device__ __forceinline__ int np_of(int qi) const { return np ? np[qi] : np_max; }
    __device__ __forceinline__ int k_of(int qi) const { return k ? k[qi] : k_max; }
};

// ------------------------------------------------------------------ probe
__global__ void k_probe_dist(DevIndexView ix, const float *__restrict__ q, float *__restrict__ dist) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = blockIdx.x * (blockDim.x >> 5) + warp;
    const int qi = blockIdx.y;
    if (c >= ix.K) return;
    const float *cr = ix.centroids + (size_t)c * ix.D;
    const float *qq = q + (size_t)qi * ix.D;
    float d = warp_eigen_sum(ix.D, [&](int i) {
        const float t = __fsub_rn(cr[i], qq[i]);
        return __fmul_rn(t, t);
    });
    if (lane == 0) dist[(size_t)qi * ix.K + c] = d;
}

// Tiled form for batches: a CTA holds kProbeQT queries in shared memory; each
// warp keeps one centroid in registers (lane (h, l) holds the elements of the
// packets p = h, h+2, ... at offset l -- Eigen's two-accumulator assignment)
// and evaluates it against every query of the tile.  Same reduction order as
// k_probe_dist (dimension a multiple of 32, so no odd packet or scalar tail).
constexpr int kProbeQT = 16, kProbeWarps = 8, kProbeRegs = 64;  // up to 64 floats per lane: dim <= 2048
__global__ void __launch_bounds__(kProbeWarps * 32) k_probe_dist_tiled(DevIndexView ix, const float *__restrict__ q,
                                                                        int nq, float *__restrict__ dist) {
    extern __shared__ float qs[];  // kProbeQT x D
    const int D = ix.D, warp = threadIdx.x >> 5, lane = threadIdx.x & 31, l = lane & 15, h = lane >> 4;
    const int q0 = blockIdx.y * kProbeQT, nqt = min(kProbeQT, nq - q0);
    for (int i = threadIdx.x; i < nqt * D; i += blockDim.x) qs[i] = q[(size_t)q0 * D + i];
    __syncthreads();
    const int npk = D / 32;  // packets per lane
    for (int c = blockIdx.x * kProbeWarps + warp; c < ix.K; c += gridDim.x * kProbeWarps) {
        const float *cr = ix.centroids + (size_t)c * D;
        float cv[kProbeRegs];
#pragma unroll
        for (int k = 0; k < kProbeRegs; ++k)
            if (k < npk) cv[k] = cr[16 * (h + 2 * k) + l];
        for (int qi = 0; qi < nqt; ++qi) {
            const float *qq = qs + qi * D;
            float acc = 0.0f;
#pragma unroll
            for (int k = 0; k < kProbeRegs; ++k)
                if (k < npk) {
                    const float t = __fsub_rn(cv[k], qq[16 * (h + 2 * k) + l]);
                    acc = k == 0 ? __fmul_rn(t, t) : __fadd_rn(acc, __fmul_rn(t, t));
                }
            acc = __fadd_rn(acc, __shfl_down_sync(kFull, acc, 16));
            acc = __fadd_rn(acc, __shfl_down_sync(kFull, acc, 8));
            acc = __fadd_rn(acc, __shfl_down_sync(kFull, acc, 4));
            acc = __fadd_rn(acc, __shfl_down_sync(kFull, acc, 2));
            acc = __fadd_rn(acc, __shfl_down_sync(kFull, acc, 1));
            if (lane == 0) dist[(size_t)(q0 + qi) * ix.K + c] = acc;
        }
    }
}

struct Cand {
    uint32_t id;
    float d;
};

// libstdc++ std::partial_sort (stl_algo.h __heap_select + __sort_heap,
// stl_heap.h __adjust_heap / __push_heap / __pop_heap), comp = operator< on
// the distance (Candidate::operator<, defines.hpp:48).
__device__ void heap_adjust(Cand *a, long hole, long len, Cand val) {
    const long top = hole;
    long sc = hole;
    while (sc < (len - 1) / 2) {
        sc = 2 * (sc + 1);
        if (a[sc].d < a[sc - 1].d) sc--;
        a[hole] = a[sc];
        hole = sc;
    }
    if ((len & 1) == 0 && sc == (len - 2) / 2) {
        sc = 2 * (sc + 1);
        a[hole] = a[sc - 1];
        hole = sc - 1;
    }
    long parent = (hole - 1) / 2;
    while (hole > top && a[parent].d < val.d) {
        a[hole] = a[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    a[hole] = val;
}

__device__ void exact_partial_sort(Cand *a, long mid, long len) {
    if (mid >= 2)
        for (long parent = (mid - 2) / 2;; --parent) {
            heap_adjust(a, parent, mid, a[parent]);
            if (parent == 0) break;
        }
    for (long i = mid; i < len; ++i)
        if (a[i].d < a[0].d) {
            Cand v = a[i];
            a[i] = a[0];
            heap_adjust(a, 0, mid, v);
        }
    for (long last = mid; last > 1;) {
        --last;
        Cand v = a[last];
        a[last] = a[0];
        heap_adjust(a, 0, last, v);
    }
}

// One radix-select step, by a whole warp: the first bin b with
// hist[0] + ... + hist[b] > rem and the count of the bins before it (what a
// sequential scan of the 256 bins finds).
__device__ __forceinline__ void select_bin(const uint32_t *hist, uint32_t rem, int &b, uint32_t &below) {
    const int lane = threadIdx.x & 31;
    uint32_t h[8], sum = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        h[i] = hist[lane * 8 + i];
        sum += h[i];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += v;
    }
    const uint32_t excl = incl - sum;
    const uint32_t m = __ballot_sync(kFull, excl <= rem && rem < incl);
    if (!m) {  // rem beyond every count: the scan runs off the end
        b = 256;
        below = __shfl_sync(kFull, incl, 31);
        return;
    }
    const int L = __ffs(m) - 1;
    int bb = 0;
    uint32_t cum = excl;
    if (lane == L) {
        int i = 0;
        for (; i < 8; ++i) {
            if (cum + h[i] > rem) break;
            cum += h[i];
        }
        bb = L * 8 + i;
    }
    b = __shfl_sync(kFull, bb, L);
    below = __shfl_sync(kFull, cum, L);
}

constexpr int kSelThreads = 1024;
constexpr int kSelMax = 1024;  // fast path handles nprobe <= 1024

__global__ void __launch_bounds__(kSelThreads) k_probe_select(const float *__restrict__ dist, int K, int nprobe_max,
                                                              uint32_t *__restrict__ probe, Cand *__restrict__ work,
                                                              int *__restrict__ fallback_count,
                                                              const uint8_t *__restrict__ only = nullptr,
                                                              const int *__restrict__ qnp = nullptr) {
    __shared__ uint32_t hist[256];
    __shared__ uint32_t s_prefix, s_mask, s_rem, s_eq, s_n;
    __shared__ unsigned long long sel[kSelMax];
    const int qi = blockIdx.x, tid = threadIdx.x;
    if (only && !only[qi]) return;  // ranked by the shortlist
    const int nprobe = qnp ? qnp[qi] : nprobe_max;  // this query's nprobe; rows are nprobe_max long
    const float *dq = dist + (size_t)qi * K;
    if (tid == 0) {
        s_prefix = 0;
        s_mask = 0;
        s_rem = (uint32_t)(nprobe - 1);
    }
    __syncthreads();
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = 24 - 8 * pass;
        for (int i = tid; i < 256; i += kSelThreads) hist[i] = 0;
        __syncthreads();
        const uint32_t prefix = s_prefix, mask = s_mask;
        for (int i = tid; i < K; i += kSelThreads) {
            const uint32_t k = fkey(dq[i]);
            if ((k & mask) == prefix) atomicAdd(&hist[(k >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (tid < 32) {
            int b;
            uint32_t cum;
            select_bin(hist, s_rem, b, cum);
            if (tid == 0) {
                s_rem = s_rem - cum;
                s_prefix = prefix | ((uint32_t)b << shift);
                s_mask = mask | (255u << shift);
                s_eq = b < 256 ? hist[b] : 0u;
                s_n = 0;
            }
        }
        __syncthreads();
    }
    const uint32_t T = s_prefix;
    const uint32_t count_lt = (uint32_t)(nprobe - 1) - s_rem;
    bool need_exact = (s_eq != 1) || nprobe > kSelMax;
    if (!need_exact) {
        for (int i = tid; i < K; i += kSelThreads) {
            const uint32_t k = fkey(dq[i]);
            if (k <= T) {
                const uint32_t pos = atomicAdd(&s_n, 1u);
                if (pos < kSelMax) sel[pos] = ((unsigned long long)k << 32) | (uint32_t)i;
            }
        }
        __syncthreads();
        const int n = (int)s_n;
        int P = 1;
        while (P < n) P <<= 1;
        for (int i = n + tid; i < P; i += kSelThreads) sel[i] = ~0ull;
        __syncthreads();
        for (int k = 2; k <= P; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = tid; i < P; i += kSelThreads) {
                    const int ixj = i ^ j;
                    if (ixj > i) {
                        const unsigned long long a = sel[i], b = sel[ixj];
                        const bool up = (i & k) == 0;
                        if ((a > b) == up) {
                            sel[i] = b;
                            sel[ixj] = a;
                        }
                    }
                }
                __syncthreads();
            }
        // equal keys inside the selection make the heap order matter
        __shared__ int s_dup;
        if (tid == 0) s_dup = (n != nprobe) || (count_lt + 1 != (uint32_t)nprobe);
        __syncthreads();
        for (int i = tid; i + 1 < n; i += kSelThreads)
            if ((sel[i] >> 32) == (sel[i + 1] >> 32)) s_dup = 1;
        __syncthreads();
        if (!s_dup) {
            for (int i = tid; i < nprobe; i += kSelThreads) probe[(size_t)qi * nprobe_max + i] = (uint32_t)(sel[i] & 0xffffffffu);
            return;
        }
        need_exact = true;
    }
    // exact fallback: the standard library's algorithm, sequentially
    if (nprobe > kSelMax) {
        if (tid == 0) {
            atomicAdd(fallback_count, 1);
            Cand *a = work + (size_t)qi * K;
            for (int i = 0; i < K; ++i) a[i] = Cand{(uint32_t)i, dq[i]};
            exact_partial_sort(a, nprobe, K);
            for (int i = 0; i < nprobe; ++i) probe[(size_t)qi * nprobe_max + i] = a[i].id;
        }
        return;
    }
    // the same steps with the heap (the first nprobe slots of the array) in
    // shared memory; the rest of the row is only ever compared against the
    // heap's top at its turn, so it streams through in coalesced chunks
    __shared__ float chunk[kSelThreads];
    Cand *heap = reinterpret_cast<Cand *>(sel);
    const int mid = nprobe;
    for (int i = tid; i < mid; i += kSelThreads) heap[i] = Cand{(uint32_t)i, dq[i]};
    __syncthreads();
    if (tid == 0) {
        atomicAdd(fallback_count, 1);
        if (mid >= 2)
            for (long parent = (mid - 2) / 2;; --parent) {
                heap_adjust(heap, parent, mid, heap[parent]);
                if (parent == 0) break;
            }
    }
    // the heap's top only shrinks, so an element not below the top at its
    // chunk's start is skipped at its own turn too: each chunk is filtered in
    // parallel against that top and thread 0 runs the steps on the rest, in order
    __shared__ int s_wcnt[kSelThreads / 32];
    __shared__ int s_list[kSelThreads];
    const int lane = tid & 31, wp = tid >> 5;
    for (int base = mid; base < K; base += kSelThreads) {
        __syncthreads();
        const float top = heap[0].d;
        const float v = base + tid < K ? dq[base + tid] : 0.0f;
        const bool in = base + tid < K && v < top;
        const uint32_t bal = __ballot_sync(kFull, in);
        if (lane == 0) s_wcnt[wp] = __popc(bal);
        chunk[tid] = v;
        __syncthreads();
        int off = 0, total = 0;
        for (int i = 0; i < kSelThreads / 32; ++i) {
            if (i < wp) off += s_wcnt[i];
            total += s_wcnt[i];
        }
        if (in) s_list[off + __popc(bal & ((1u << lane) - 1))] = tid;
        __syncthreads();
        if (tid == 0)
            for (int r = 0; r < total; ++r) {
                const int j = s_list[r];
                if (chunk[j] < heap[0].d) heap_adjust(heap, 0, mid, Cand{(uint32_t)(base + j), chunk[j]});
            }
    }
    if (tid == 0) {
        for (long last = mid; last > 1;) {
            --last;
            const Cand v = heap[last];
            heap[last] = heap[0];
            heap_adjust(heap, 0, last, v);
        }
        for (int i = 0; i < mid; ++i) probe[(size_t)qi * nprobe_max + i] = heap[i].id;
    }
}

// ------------------------------------------------------ probe: GEMM shortlist
// Batches rank centroids from inner products q.c computed by a BF16
// tensor-core GEMM (probe_gemm.cu).  Each approximate distance a = |q|^2 +
// |c|^2 - 2 q.c gets a rigorous bound b on its distance from the reference's
// float distance (operands rounded to BF16 are within 2^-9 of their FP32
// values, so |q.c error| <= (2^-8 + 2^-18 + accumulation) |q||c|; the norms and
// the reference's own sum add (2D + 32) * 2^-24 (|q| + |c|)^2).  Every centroid of the exact top-nprobe has
// a - b <= T, T the nprobe-th smallest a + b, so only those centroids get the
// exact Eigen-order distance and the ranking is the exact one.  A query with
// equal distances among its first nprobe + 1 (where the standard library's
// heap order decides), a non-finite value or more than kShortCap centroids on
// its shortlist is ranked by the full exact path instead.
constexpr int kShortThreads = 512;
constexpr int kShortCap = 1024;  // shortlist capacity (more: the full exact path); keeps 2 CTAs per SM
constexpr int kGemmMinQueries = 64;  // smaller calls rank with the exact kernels directly

constexpr int kShortKeys = 16384;    // clusters whose upper-bound keys the shortlist keeps in shared memory

// |c|^2 and |c| of every centroid (any summation order: only the bounds use them)
__global__ void k_cnorm2(DevIndexView ix, float2 *__restrict__ cn) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= ix.K) return;
    const float *cr = ix.centroids + (size_t)warp * ix.D;
    float a = 0.0f;
    for (int i = lane; i < ix.D; i += 32) a += cr[i] * cr[i];
    for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(kFull, a, o);
    if (lane == 0) cn[warp] = make_float2(a, sqrtf(a));
}

struct ShortBound {
    float e1, e2;  // b = e1 |q||c| + e2 (|q| + |c|)^2
};

__device__ __forceinline__ void approx_bounds(float qn2, float qn, float ip, float2 cnn, const ShortBound &sb, float &lo,
                                              float &hi) {
    const float cn2 = cnn.x, cn = cnn.y;
    const float a = (qn2 + cn2) - 2.0f * ip;
    const float s = qn + cn;
    const float b = (sb.e1 * qn * cn + sb.e2 * s * s) * 1.01f + 1e-30f;
    lo = a - b;
    hi = a + b;
}

__global__ void __launch_bounds__(kShortThreads) k_probe_shortlist(DevIndexView ix, const float *__restrict__ q,
                                                                   const float *__restrict__ ip,
                                                                   const float2 *__restrict__ cn2, ShortBound sb,
                                                                   int nprobe_max, const int *__restrict__ qnp,
                                                                   uint32_t *__restrict__ probe,
                                                                   uint8_t *__restrict__ full, int *__restrict__ fb_list,
                                                                   int *__restrict__ fb_count,
                                                                   unsigned long long *__restrict__ counters,
                                                                   const int *__restrict__ ip_err, int keep_keys) {
    extern __shared__ __align__(16) char smem_raw[];
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(smem_raw);  // [kShortCap]
    uint32_t *cand = reinterpret_cast<uint32_t *>(keys + kShortCap);             // [kShortCap]
    float *qs = reinterpret_cast<float *>(cand + kShortCap);                      // [D]
    uint32_t *hk = reinterpret_cast<uint32_t *>(qs + ix.D);                       // [K] when keep_keys
    const bool keep = keep_keys != 0;
    __shared__ uint32_t hist[256];
    __shared__ uint32_t tmin[kShortThreads];
    __shared__ uint32_t s_prefix, s_mask, s_rem, s_n;
    __shared__ int s_bad;
    __shared__ float s_red[kShortThreads / 32];
    const int qi = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int K = ix.K, D = ix.D;
    const int nprobe = qnp ? qnp[qi] : nprobe_max;
    const float *ipq = ip + (size_t)qi * K;
    float a = 0.0f;
    for (int i = tid; i < D; i += kShortThreads) {
        const float v = q[(size_t)qi * D + i];
        qs[i] = v;
        a += v * v;
    }
    for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(kFull, a, o);
    if (lane == 0) s_red[warp] = a;
    if (tid == 0) {
        s_prefix = 0;
        s_mask = 0;
        s_rem = (uint32_t)(nprobe - 1);
        s_n = 0;
        s_bad = 0;
    }
    __syncthreads();
    float qn2 = 0.0f;
    for (int i = 0; i < kShortThreads / 32; ++i) qn2 += s_red[i];
    const float qn = sqrtf(qn2);
    // T: the nprobe-th smallest upper end (radix select on the order-preserving
    // keys).  For nprobe <= threads / 2, each thread contributes the smallest
    // upper end of its strided share of the centroids and T is the nprobe-th
    // smallest of those: the nprobe-th smallest of a subset of the upper ends is
    // at least the nprobe-th smallest of all, so the shortlist below still holds
    // every centroid of the exact top-nprobe (it may hold a few more).
    const bool by_thread = nprobe <= kShortThreads / 2;
    if (by_thread) {
        uint32_t m = 0xffffffffu;
        for (int c = tid; c < K; c += kShortThreads) {
            float lo, hi;
            approx_bounds(qn2, qn, ipq[c], cn2[c], sb, lo, hi);
            if (!(isfinite(lo) && isfinite(hi))) s_bad = 1;
            m = min(m, fkey(hi));
        }
        tmin[tid] = m;
    }
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = 24 - 8 * pass;
        for (int i = tid; i < 256; i += kShortThreads) hist[i] = 0;
        __syncthreads();
        const uint32_t prefix = s_prefix, mask = s_mask;
        if (by_thread) {
            const uint32_t k = tmin[tid];
            if ((k & mask) == prefix) atomicAdd(&hist[(k >> shift) & 255u], 1u);
        } else {
            for (int c = tid; c < K; c += kShortThreads) {
                uint32_t k;
                if (pass == 0 || !keep) {
                    float lo, hi;
                    approx_bounds(qn2, qn, ipq[c], cn2[c], sb, lo, hi);
                    if (pass == 0 && !(isfinite(lo) && isfinite(hi))) s_bad = 1;
                    k = fkey(hi);
                    if (keep) hk[c] = k;
                } else {
                    k = hk[c];
                }
                if ((k & mask) == prefix) atomicAdd(&hist[(k >> shift) & 255u], 1u);
            }
        }
        __syncthreads();
        if (tid < 32) {
            int b;
            uint32_t cum;
            select_bin(hist, s_rem, b, cum);
            if (tid == 0) {
                s_rem = s_rem - cum;
                s_prefix = prefix | ((uint32_t)b << shift);
                s_mask = mask | (255u << shift);
            }
        }
        __syncthreads();
    }
    const float T = key_to_float(s_prefix);
    if (*ip_err) s_bad = 1;  // the inner products are incomplete: the full exact path ranks every query
    // the shortlist: lower end not above T
    if (!s_bad)
        for (int c = tid; c < K; c += kShortThreads) {
            float lo, hi;
            approx_bounds(qn2, qn, ipq[c], cn2[c], sb, lo, hi);
            if (lo <= T) {
                const uint32_t pos = atomicAdd(&s_n, 1u);
                if (pos < kShortCap) cand[pos] = (uint32_t)c;
            }
        }
    __syncthreads();
    const int n = (int)s_n;
    if (s_bad || n > kShortCap) {
        if (tid == 0) {
            full[qi] = 1;
            fb_list[atomicAdd(fb_count, 1)] = qi;
            if (counters) atomicAdd(counters + 5, 1ull);
            if (counters) atomicAdd(counters + 4, (unsigned long long)K);
        }
        return;
    }
    // exact distances of the shortlist, in the reference's order (as k_probe_dist)
    for (int i = warp; i < n; i += kShortThreads / 32) {
        const uint32_t c = cand[i];
        const float *cr = ix.centroids + (size_t)c * D;
        const float d = warp_eigen_sum(D, [&](int e) {
            const float t = __fsub_rn(cr[e], qs[e]);
            return __fmul_rn(t, t);
        });
        if (lane == 0) {
            if (d != d) s_bad = 1;
            keys[i] = ((unsigned long long)fkey(d) << 32) | c;
        }
    }
    int P = 1;
    while (P < n) P <<= 1;
    for (int i = n + tid; i < P; i += kShortThreads) keys[i] = ~0ull;
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < P; i += kShortThreads) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const unsigned long long x = keys[i], y = keys[ixj];
                    if ((x > y) == ((i & k) == 0)) {
                        keys[i] = y;
                        keys[ixj] = x;
                    }
                }
            }
            __syncthreads();
        }
    // equal distances among the first nprobe + 1 leave the order to the heap
    const int m = min(n, nprobe + 1);
    for (int i = tid; i + 1 < m; i += kShortThreads)
        if ((keys[i] >> 32) == (keys[i + 1] >> 32)) s_bad = 1;
    __syncthreads();
    if (s_bad || n < nprobe) {
        if (tid == 0) {
            full[qi] = 1;
            fb_list[atomicAdd(fb_count, 1)] = qi;
            if (counters) atomicAdd(counters + 6, 1ull);
            if (counters) atomicAdd(counters + 4, (unsigned long long)K);
        }
        return;
    }
    for (int i = tid; i < nprobe; i += kShortThreads) probe[(size_t)qi * nprobe_max + i] = (uint32_t)(keys[i] & 0xffffffffu);
    if (tid == 0) {
        full[qi] = 0;
        if (counters) atomicAdd(counters + 4, (unsigned long long)n);
    }
}

// Exact distances to every centroid for the queries the shortlist handed back
// (a grid-stride loop over (query, group of 8 centroids)).
__global__ void k_probe_dist_list(DevIndexView ix, const float *__restrict__ q, float *__restrict__ dist,
                                  const int *__restrict__ fb_list, const int *__restrict__ fb_count) {
    const int nfb = *fb_count;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    const int groups = (ix.K + wpb - 1) / wpb;
    for (long w = blockIdx.x; w < (long)nfb * groups; w += gridDim.x) {
        const int qi = fb_list[w / groups], c = (int)(w % groups) * wpb + warp;
        if (c >= ix.K) continue;
        const float *cr = ix.centroids + (size_t)c * ix.D;
        const float *qq = q + (size_t)qi * ix.D;
        const float d = warp_eigen_sum(ix.D, [&](int i) {
            const float t = __fsub_rn(cr[i], qq[i]);
            return __fmul_rn(t, t);
        });
        if (lane == 0) dist[(size_t)qi * ix.K + c] = d;
    }
}

// ------------------------------------------------------------------ query prep
__global__ void k_qprep(DevIndexView ix, const float *__restrict__ q, float m, float *__restrict__ qrot,
                        float *__restrict__ prune) {
    extern __shared__ float cq[];
    const int s = blockIdx.x, qi = blockIdx.y;
    const SegDev &g = ix.seg[s];
    const int dim = g.dim, qoff = g.qoff;
    for (int i = threadIdx.x; i < dim; i += blockDim.x) {
        const int gi = qoff + i;
        cq[i] = gi < ix.D ? q[(size_t)qi * ix.D + gi] : 0.0f;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const float *var = ix.var + qoff;
        const float v2 = warp_eigen_sum(dim, [&](int i) { return __fmul_rn(var[i], __fmul_rn(cq[i], cq[i])); });
        if (threadIdx.x == 0) prune[(size_t)qi * ix.S + s] = __fmul_rn(sqrtf(v2), m);
    }
    float *out = qrot + (size_t)qi * ix.Dtot + qoff;
    if (!g.P) {
        for (int i = threadIdx.x; i < dim; i += blockDim.x) out[i] = cq[i];
        return;
    }
    // Eigen general_matrix_vector_product<ColMajor> (GeneralMatrixVector.h:108-300):
    // per output, FMA chains over blocks of 16 inputs (one block if dim < 128).
    const int bc = dim < 128 ? dim : 16;
    for (int i = threadIdx.x; i < dim; i += blockDim.x) {
        float res = 0.0f;
        for (int j2 = 0; j2 < dim; j2 += bc) {
            float c = 0.0f;
            const int je = min(j2 + bc, dim);
            for (int j = j2; j < je; ++j) c = fmaf(g.P[(size_t)j * dim + i], cq[j], c);
            res = fmaf(c, 1.0f, res);
        }
        out[i] = res;
    }
}

// ------------------------------------------------------------------ LUT

// 16 float LUT entries of one 4-dim codebook: fastscan::pack_lut (fastscan.hpp:236-248),
// entry j = entry[j - lowbit(j)] + q[kPos[j]].
__device__ __forceinline__ void lut_entries(const float *__restrict__ qq, float *t) {
    t[0] = 0.0f;
#pragma unroll
    for (int j = 1; j < 16; ++j) {
        const int lb = j & -j, pos = lb == 1 ? 3 : lb == 2 ? 2 : lb == 4 ? 1 : 0;  // kPos[j] (fastscan.hpp:22-39)
        t[j] = __fadd_rn(t[j - lb], qq[pos]);
    }
}

// FastScan sum of one vector (this lane) of block gb: sum over codebooks of
// LUT_u16[cb][nibble] (accumulate_hacc, fastscan_highacc.hpp:66-139, exact
// for dim <= 2048), then Lut::compFastIP's float epilogue and the L2 form of
// CaqCluEstimator::compFastDist (caq_estimator.hpp:148-179).
__device__ __forceinline__ float fast_est(const SegDev &g, const uint16_t *__restrict__ lut, const SegScal &sc,
                                          int64_t gb, int lane, float onorm, float &ipx) {
    const int nc = g.dim / 64;
    const uint2 *cp = g.codes + (size_t)gb * nc * 32 + lane;
    int sum = 0;
#pragma unroll 4
    for (int c8 = 0; c8 < nc; ++c8) {
        const uint2 w = cp[(size_t)c8 * 32];
        const char *L = reinterpret_cast<const char *>(lut + c8 * 256);
        // byte k of these holds 2 x (high / low nibble of code byte k): the byte
        // offset of the entry within its 16-entry u16 table
        const uint32_t hx = (w.x >> 3) & 0x1E1E1E1Eu, lx = (w.x << 1) & 0x1E1E1E1Eu;
        const uint32_t hy = (w.y >> 3) & 0x1E1E1E1Eu, ly = (w.y << 1) & 0x1E1E1E1Eu;
#pragma unroll
        for (int j = 0; j < 4; ++j)
            sum += *reinterpret_cast<const uint16_t *>(L + (2 * j) * 32 + __byte_perm(hx, 0u, 0x4440u | j)) +
                   *reinterpret_cast<const uint16_t *>(L + (2 * j + 1) * 32 + __byte_perm(lx, 0u, 0x4440u | j));
#pragma unroll
        for (int j = 0; j < 4; ++j)
            sum += *reinterpret_cast<const uint16_t *>(L + (8 + 2 * j) * 32 + __byte_perm(hy, 0u, 0x4440u | j)) +
                   *reinterpret_cast<const uint16_t *>(L + (8 + 2 * j + 1) * 32 + __byte_perm(ly, 0u, 0x4440u | j));
    }
    float t = __fmul_rn((float)sum, sc.delta);
    t = __fadd_rn(t, sc.sum_vl);
    ipx = t;
    float f = __fmul_rn(__fsub_rn(t, sc.c1), sc.c2);
    f = __fmul_rn(f, onorm);
    return maxps(0.0f, __fadd_rn(__fmul_rn(onorm, onorm), __fsub_rn(sc.q_l2sqr, f)));
}

__device__ __forceinline__ float vars_est(const SegScal &sc, float onorm) {
    return maxps(0.0f, __fadd_rn(__fmul_rn(onorm, onorm), sc.vfac));
}

// ResultPool::insert / distk (utils/pool.hpp:17-49), L2
__device__ __forceinline__ void pool_insert(uint32_t *ids, float *d, int &size, int cap, uint32_t u, float dist) {
    if (size == cap && dist > d[size - 1]) return;
    int lo = 0, len = size;
    while (len > 1) {
        const int half = len >> 1;
        len -= half;
        lo += (d[lo + half - 1] < dist) * half;
    }
    if (lo < size && d[lo] < dist) lo++;
    for (int i = size; i > lo; --i) {
        ids[i] = ids[i - 1];
        d[i] = d[i - 1];
    }
    ids[lo] = u;
    d[lo] = dist;
    size += (size < cap);
}

// k_qprep for a few queries, spread for latency: in Eigen's GEMV order the
// 16-input block sums c_b of an output are independent (only their fold
// res = fma(c_b, 1, res) runs in block order), so a CTA takes 32 outputs of
// one (segment, query), its warps compute the block sums (lane = output, a
// 16-step chain each), and warp 0 folds them in order.  Bit-identical to
// k_qprep; the prune bound comes from the CTA holding the first 32 outputs.
constexpr int kQprepOut = 32;
__global__ void __launch_bounds__(256) k_qprep_small(DevIndexView ix, const float *__restrict__ q, float m,
                                                     float *__restrict__ qrot, float *__restrict__ prune) {
    extern __shared__ __align__(16) float qsm[];  // [dim] query slice, then [dim / 16][32] block sums
    const int s = blockIdx.x, qi = blockIdx.y, o0 = blockIdx.z * kQprepOut;
    const SegDev &g = ix.seg[s];
    const int dim = g.dim, qoff = g.qoff;
    if (o0 >= dim) return;
    float *cq = qsm, *part = qsm + dim;
    for (int i = threadIdx.x; i < dim; i += blockDim.x) {
        const int gi = qoff + i;
        cq[i] = gi < ix.D ? q[(size_t)qi * ix.D + gi] : 0.0f;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, i = o0 + lane;
    if (blockIdx.z == 0 && warp == 1) {
        const float *var = ix.var + qoff;
        const float v2 = warp_eigen_sum(dim, [&](int e) { return __fmul_rn(var[e], __fmul_rn(cq[e], cq[e])); });
        if (lane == 0) prune[(size_t)qi * ix.S + s] = __fmul_rn(sqrtf(v2), m);
    }
    float *out = qrot + (size_t)qi * ix.Dtot + qoff;
    if (!g.P) {
        if (warp == 0 && i < dim) out[i] = cq[i];
        return;
    }
    const int bc = dim < 128 ? dim : 16, nbk = (dim + bc - 1) / bc;
    for (int b = warp; b < nbk; b += blockDim.x >> 5) {
        float c = 0.0f;
        const int j2 = b * bc, je = min(j2 + bc, dim);
        if (i < dim)
            for (int j = j2; j < je; ++j) c = fmaf(g.P[(size_t)j * dim + i], cq[j], c);
        part[b * kQprepOut + lane] = c;
    }
    __syncthreads();
    if (warp == 0 && i < dim) {
        float res = 0.0f;
        for (int b = 0; b < nbk; ++b) res = fmaf(part[b * kQprepOut + lane], 1.0f, res);
        out[i] = res;
    }
}

// k_qprep for a tile of kQprepQT queries per CTA: each P element is read once
// for the whole tile and drives kQprepQT independent chains, each in exactly
// k_qprep's order (so the outputs are bit-identical); L2 traffic for the
// rotations drops by the tile size.  A CTA computes kQprepSlice outputs (one
// per thread; blockIdx.z picks the slice), and the P column of the next
// 16-input block is loaded while the current block's chains run.
constexpr int kQprepQT = 16;
constexpr int kQprepSlice = 256;
__global__ void __launch_bounds__(kQprepSlice) k_qprep_tiled(DevIndexView ix, const float *__restrict__ q, int nq,
                                                             float m, float *__restrict__ qrot,
                                                             float *__restrict__ prune) {
    extern __shared__ __align__(16) float cqs[];  // [kQprepQT][dim]
    const int s = blockIdx.x, q0 = blockIdx.y * kQprepQT, nqt = min(kQprepQT, nq - q0);
    const SegDev &g = ix.seg[s];
    const int dim = g.dim, qoff = g.qoff;
    const int i = blockIdx.z * kQprepSlice + threadIdx.x;
    if (blockIdx.z * kQprepSlice >= dim) return;
    for (int e = threadIdx.x; e < kQprepQT * dim; e += blockDim.x) {
        const int t = e / dim, ii = e - t * dim, gi = qoff + ii;
        cqs[e] = (t < nqt && gi < ix.D) ? q[(size_t)(q0 + t) * ix.D + gi] : 0.0f;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5;
    if (blockIdx.z == 0)
        for (int t = warp; t < nqt; t += blockDim.x >> 5) {
            const float *cq = cqs + t * dim, *var = ix.var + qoff;
            const float v2 = warp_eigen_sum(dim, [&](int k) { return __fmul_rn(var[k], __fmul_rn(cq[k], cq[k])); });
            if ((threadIdx.x & 31) == 0) prune[(size_t)(q0 + t) * ix.S + s] = __fmul_rn(sqrtf(v2), m);
        }
    if (i >= dim) return;
    if (!g.P) {
        for (int t = 0; t < nqt; ++t) qrot[(size_t)(q0 + t) * ix.Dtot + qoff + i] = cqs[t * dim + i];
        return;
    }
    float res[kQprepQT], c[kQprepQT];
#pragma unroll
    for (int t = 0; t < kQprepQT; ++t) res[t] = 0.0f;
    if (dim < 128) {  // one block of `dim` inputs (dims are multiples of 64)
#pragma unroll
        for (int t = 0; t < kQprepQT; ++t) c[t] = 0.0f;
        for (int j = 0; j < dim; j += 4) {
            const float p0 = g.P[(size_t)j * dim + i], p1 = g.P[(size_t)(j + 1) * dim + i];
            const float p2 = g.P[(size_t)(j + 2) * dim + i], p3 = g.P[(size_t)(j + 3) * dim + i];
#pragma unroll
            for (int t = 0; t < kQprepQT; ++t) {
                const float4 v = *reinterpret_cast<const float4 *>(cqs + t * dim + j);
                c[t] = fmaf(p0, v.x, c[t]);
                c[t] = fmaf(p1, v.y, c[t]);
                c[t] = fmaf(p2, v.z, c[t]);
                c[t] = fmaf(p3, v.w, c[t]);
            }
        }
#pragma unroll
        for (int t = 0; t < kQprepQT; ++t) res[t] = fmaf(c[t], 1.0f, res[t]);
    } else {  // blocks of 16 inputs, the next block's P column in flight
        float pc[16], pn[16];
#pragma unroll
        for (int jj = 0; jj < 16; ++jj) pc[jj] = g.P[(size_t)jj * dim + i];
        for (int j2 = 0; j2 < dim; j2 += 16) {
            if (j2 + 16 < dim) {
#pragma unroll
                for (int jj = 0; jj < 16; ++jj) pn[jj] = g.P[(size_t)(j2 + 16 + jj) * dim + i];
            }
#pragma unroll
            for (int t = 0; t < kQprepQT; ++t) c[t] = 0.0f;
#pragma unroll
            for (int jj = 0; jj < 16; jj += 4) {
#pragma unroll
                for (int t = 0; t < kQprepQT; ++t) {
                    const float4 v = *reinterpret_cast<const float4 *>(cqs + t * dim + j2 + jj);
                    c[t] = fmaf(pc[jj], v.x, c[t]);
                    c[t] = fmaf(pc[jj + 1], v.y, c[t]);
                    c[t] = fmaf(pc[jj + 2], v.z, c[t]);
                    c[t] = fmaf(pc[jj + 3], v.w, c[t]);
                }
            }
#pragma unroll
            for (int t = 0; t < kQprepQT; ++t) res[t] = fmaf(c[t], 1.0f, res[t]);
#pragma unroll
            for (int jj = 0; jj < 16; ++jj) pc[jj] = pn[jj];
        }
    }
#pragma unroll
    for (int t = 0; t < kQprepQT; ++t)
        if (t < nqt) qrot[(size_t)(q0 + t) * ix.Dtot + qoff + i] = res[t];
}

// ------------------------------------------------------------------ scan
struct ScanSmem {
    // laid out in dynamic shared memory by scan_smem_layout()
    uint16_t *lut;
    float *qres;
    SegScal *scal;
    float *cd, *ipx, *part, *cur, *stage;
    uint32_t *cmask;
    int *nstage;
    uint32_t *pool_id;
    float *pool_d;
    uint32_t *mm;     // per segment LUT min / max keys
    uint8_t *xbuf;    // per half-warp ex-code staging
    int xstride;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

__host__ __device__ inline size_t scan_smem_bytes(int Dtot, int S, int topk, int xstride) {
    size_t b = 0;
    b += align16(sizeof(uint32_t) * 2 * S);
    b += align16((size_t)2 * kScanWarps * xstride);
    b += align16(sizeof(uint16_t) * 4 * (size_t)Dtot);
    b += align16(sizeof(float) * Dtot);
    b += align16(sizeof(SegScal) * S);
    b += 2 * align16(sizeof(float) * kTileB * S * 32);  // cd (= part), ipx
    b += align16(sizeof(float) * kTileB * 32);          // cur
    b += align16(sizeof(float) * kTileB * (S + 1));     // stage minima
    b += align16(sizeof(uint32_t) * kTileB);
    b += align16(sizeof(int) * kTileB);
    b += align16(sizeof(uint32_t) * (topk + 1));
    b += align16(sizeof(float) * (topk + 1));
    return b;
}

__device__ ScanSmem scan_smem_layout(char *base, int Dtot, int S, int topk, int xstride) {
    ScanSmem s;
    size_t o = 0;
    s.mm = (uint32_t *)(base + o);
    o += align16(sizeof(uint32_t) * 2 * S);
    s.xbuf = (uint8_t *)(base + o);
    s.xstride = xstride;
    o += align16((size_t)2 * kScanWarps * xstride);
    s.lut = (uint16_t *)(base + o);
    o += align16(sizeof(uint16_t) * 4 * (size_t)Dtot);
    s.qres = (float *)(base + o);
    o += align16(sizeof(float) * Dtot);
    s.scal = (SegScal *)(base + o);
    o += align16(sizeof(SegScal) * S);
    s.cd = (float *)(base + o);
    o += align16(sizeof(float) * kTileB * S * 32);
    s.ipx = (float *)(base + o);
    o += align16(sizeof(float) * kTileB * S * 32);
    // A candidate's partial replaces its estimate in place: the accurate pass
    // reads cd[i] and writes part[i] in the same thread, and nothing reads a
    // candidate's estimate afterwards (the replay and the split pass's records
    // read partials of candidate lanes only).
    s.part = s.cd;
    s.cur = (float *)(base + o);
    o += align16(sizeof(float) * kTileB * 32);
    s.stage = (float *)(base + o);
    o += align16(sizeof(float) * kTileB * (S + 1));
    s.cmask = (uint32_t *)(base + o);
    o += align16(sizeof(uint32_t) * kTileB);
    s.nstage = (int *)(base + o);
    o += align16(sizeof(int) * kTileB);
    s.pool_id = (uint32_t *)(base + o);
    o += align16(sizeof(uint32_t) * (topk + 1));
    s.pool_d = (float *)(base + o);
    return s;
}

// ---- pieces of Lut::prepare (lut.hpp:60-87) shared by the in-CTA preparation
// (prepare_cluster) and the batched one (k_lut), so both give the same bits.
// The quantizer's scale from the segment's LUT min / max keys.
__device__ __forceinline__ void seg_quant_scalars(uint32_t kmin, uint32_t kmax, SegScal &sc) {
    const float vl = key_to_float(kmin), vr = key_to_float(kmax);
    const float delta = (float)__ddiv_rn((double)__fsub_rn(vr, vl), 65536.0 - 0.01);
    sc.delta = delta;
    sc.rdelta = __frcp_rn(delta);
    sc.vl = vl;
}

// compFastIP's epilogue constants (sum_q, q_l2sqr, vl and delta already set).
__device__ __forceinline__ void seg_epilogue_scalars(const SegDev &g, float prune_s, SegScal &sc) {
    const int ncb = g.dim / 4;
    sc.sum_vl = (float)__dmul_rn(__dadd_rn((double)sc.vl, __dmul_rn(0.5, (double)sc.delta)), (double)(float)ncb);
    sc.q_l2norm = sqrtf(sc.q_l2sqr);
    sc.c1 = (float)__dsub_rn(__dmul_rn(0.5, (double)sc.sum_q), (double)__fmul_rn(0.58f, sc.q_l2norm));
    sc.c2 = g.c2;
    sc.vfac = __fsub_rn(sc.q_l2sqr, __fmul_rn(2.0f, prune_s));
}

// Float entry j of one codebook in lut_entries' order: entry j = entry[j -
// lowbit(j)] + q[kPos[lowbit(j)]], so the dims of j's bits are added from the
// highest bit down (kPos of bit b is 3 - b).
__device__ __forceinline__ float lut_entry_at(const float *qq, int j) {
    float t = 0.0f;
    for (int b = 3; b >= 0; --b)
        if ((j >> b) & 1) t = __fadd_rn(t, qq[3 - b]);
    return t;
}

// The 16 u16 entries of one codebook (4 residual dims at qq), 32 bytes at dst.
// Every entry takes the multiply first; the few that it cannot settle (about 3%)
// are divided afterwards and stored over it, in a loop whose trip count is the
// lane's own number of such entries, so a warp runs a handful of divisions per
// codebook instead of one per entry that any lane needs.
__device__ __forceinline__ void quant_codebook(const float *qq, float vl, float delta, float rd, uint16_t *dst) {
    float t[16];
    lut_entries(qq, t);
    uint32_t packed[8];
    uint32_t slow = 0;
#pragma unroll
    for (int j = 0; j < 16; j += 2) {
        bool oa, ob;
        const uint32_t a = lut_quant_fast(__fsub_rn(t[j], vl), rd, oa);
        const uint32_t b = lut_quant_fast(__fsub_rn(t[j + 1], vl), rd, ob);
        slow |= (oa ? 0u : 1u << j) | (ob ? 0u : 2u << j);
        packed[j / 2] = a | (b << 16);
    }
    uint4 *d = reinterpret_cast<uint4 *>(dst);
    d[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
    d[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
    while (slow) {  // same thread, same address: the later store wins
        const int j = __ffs(slow) - 1;
        slow &= slow - 1;
        dst[j] = (uint16_t)(int)__fdiv_rn(__fsub_rn(lut_entry_at(qq, j), vl), delta);
    }
}

// Min and max keys of one codebook's float entries.
__device__ __forceinline__ void codebook_keys(const float *qq, uint32_t &kmin, uint32_t &kmax) {
    float t[16];
    lut_entries(qq, t);
    float lo = t[0], hi = t[0];
#pragma unroll
    for (int j = 1; j < 16; ++j) {
        lo = fminf(lo, t[j]);
        hi = fmaxf(hi, t[j]);
    }
    kmin = fkey(lo);
    kmax = fkey(hi);
}

// Lut::prepare (lut.hpp:60-87) for every segment of cluster c, spread over the
// whole CTA: residual query, its Eigen-order sum and squared norm, the float
// LUT's min / max, delta = (max-min)/(65536-0.01) in double, the u16 LUT
// trunc((entry-min)/delta), and the epilogue constants of compFastIP.
// t_first > 0: only threads [t_first, blockDim.x) take part (whole warps),
// synchronising on named barrier `bar` instead of __syncthreads.
__device__ void prepare_cluster(const DevIndexView &ix, const float *__restrict__ qrot, const float *__restrict__ prune,
                                int c, ScanSmem &sm, int t_first = 0, int bar = 0) {
    const int tid = (int)threadIdx.x - t_first, nt = (int)blockDim.x - t_first, warp = tid >> 5, lane = tid & 31;
    const int S = ix.S;
    auto sync = [&]() {
        if (bar) asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nt) : "memory");
        else __syncthreads();
    };
    for (int i = tid; i < ix.Dtot; i += nt) {
        int s = 0;
        while (s + 1 < S && i >= ix.seg[s + 1].qoff) ++s;
        const SegDev &g = ix.seg[s];
        sm.qres[i] = __fsub_rn(qrot[i], g.cent[(size_t)c * g.dim + (i - g.qoff)]);
    }
    if (tid < S) {
        sm.mm[2 * tid] = 0xffffffffu;  // min key
        sm.mm[2 * tid + 1] = 0u;       // max key
    }
    sync();
    for (int t = warp; t < 2 * S; t += nt / 32) {
        const int s = t >> 1;
        const float *qr = sm.qres + ix.seg[s].qoff;
        const float r = (t & 1) ? warp_eigen_sum(ix.seg[s].dim, [&](int i) { return __fmul_rn(qr[i], qr[i]); })
                                : warp_eigen_sum(ix.seg[s].dim, [&](int i) { return qr[i]; });
        if (lane == 0) {
            if (t & 1) sm.scal[s].q_l2sqr = r;
            else sm.scal[s].sum_q = r;
        }
    }
    const int ncb_all = ix.Dtot / 4;
    for (int cb0 = 0; cb0 < ncb_all; cb0 += nt) {  // warp-uniform trip count
        const int cb = cb0 + tid;
        int s = -1;
        uint32_t kmin = 0xffffffffu, kmax = 0u;
        if (cb < ncb_all) {
            s = 0;
            while (s + 1 < S && cb * 4 >= ix.seg[s + 1].qoff) ++s;
            codebook_keys(sm.qres + cb * 4, kmin, kmax);
        }
        // one shared atomic per segment present in the warp
        const unsigned grp = __match_any_sync(kFull, s);
        kmin = __reduce_min_sync(grp, kmin);
        kmax = __reduce_max_sync(grp, kmax);
        if (s >= 0 && lane == __ffs(grp) - 1) {
            atomicMin(&sm.mm[2 * s], kmin);
            atomicMax(&sm.mm[2 * s + 1], kmax);
        }
    }
    sync();
    if (tid < S) seg_quant_scalars(sm.mm[2 * tid], sm.mm[2 * tid + 1], sm.scal[tid]);  // what the quantizer needs
    sync();
    if (tid >= nt - S) {  // the epilogue constants, beside the quantization (the last warp's last lanes)
        const int s = tid - (nt - S);
        seg_epilogue_scalars(ix.seg[s], prune[s], sm.scal[s]);
    }
    for (int cb = tid; cb < ncb_all; cb += nt) {
        int s = 0;
        while (s + 1 < S && cb * 4 >= ix.seg[s + 1].qoff) ++s;
        const SegScal &sc = sm.scal[s];
        quant_codebook(sm.qres + cb * 4, sc.vl, sc.delta, sc.rdelta, sm.lut + cb * 16);
    }
    sync();
}

// Output of the batched preparation (k_lut) for the first `slots` entries of the
// split list; other entries (and null members) build each cluster's state in
// the scan CTA.
struct Prepared {
    const uint16_t *lut = nullptr;
    const SegScal *scal = nullptr;
    int np_max = 0;
    int slots = 0;
    __device__ __forceinline__ bool has(int slot) const { return lut != nullptr && slot < slots; }
    __device__ __forceinline__ const uint16_t *lut_of(int slot, int p, int Dtot) const {
        return lut + ((size_t)slot * np_max + p) * 4 * Dtot;
    }
    __device__ __forceinline__ const SegScal *scal_of(int slot, int p, int S) const {
        return scal + ((size_t)slot * np_max + p) * S;
    }
};

// ---- batched preparation: the LUT and scalars of the (query, probe) pairs of
// the first `slots` entries of a list (the split pass's), one warp per pair.
// Pair i = slot * np_max + probe; its LUT is 4 * Dtot u16 at lut + i * 4 * Dtot
// (the layout of ScanSmem::lut), its scalars S SegScal at scal + i * S.  Work
// item w is list entry w / np_max (entries at or past *nlist are none) and
// probe w % np_max.  Pairs past a query's nprobe and pairs of empty clusters
// are not written (no scan reads them).
constexpr int kLutWarps = 8;
__global__ void __launch_bounds__(kLutWarps * 32) k_lut(DevIndexView ix, const uint32_t *__restrict__ probe,
                                                        QueryShape qsh, const int *__restrict__ qlist,
                                                        const int *__restrict__ nlist, int cap,
                                                        const uint8_t *__restrict__ skip,
                                                        const float *__restrict__ qrot_all,
                                                        const float *__restrict__ prune_all, uint16_t *__restrict__ lut,
                                                        SegScal *__restrict__ scal) {
    extern __shared__ __align__(16) float k_lut_qres[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t w = (int64_t)blockIdx.x * kLutWarps + warp;
    const int slot = (int)(w / qsh.np_max), p = (int)(w - (int64_t)slot * qsh.np_max);
    if (slot >= (qlist ? min(*nlist, cap) : cap)) return;  // whole warp
    const int qi = qlist ? qlist[slot] : slot;  // no list: every query, entry = query
    if (p >= qsh.np_of(qi) || (skip && skip[qi])) return;
    const int64_t pair = (int64_t)slot * qsh.np_max + p;
    const int c = (int)probe[(size_t)qi * qsh.np_max + p];
    if (ix.blk_off[c + 1] == ix.blk_off[c]) return;
    float *qres = k_lut_qres + (size_t)warp * ix.Dtot;
    const float *qrot = qrot_all + (size_t)qi * ix.Dtot;
    for (int s = 0; s < ix.S; ++s) {
        const SegDev &g = ix.seg[s];
        const float *cent = g.cent + (size_t)c * g.dim;
        for (int i = lane; i < g.dim; i += 32) qres[g.qoff + i] = __fsub_rn(qrot[g.qoff + i], cent[i]);
    }
    __syncwarp();
    uint16_t *L = lut + pair * 4 * ix.Dtot;
    // segment s's sums and LUT min / max keys end in lane s, so the scalar steps
    // (FP64) of all segments run at once, one lane each
    SegScal sc;
    uint32_t my_min = 0xffffffffu, my_max = 0u;
    for (int s = 0; s < ix.S; ++s) {
        const SegDev &g = ix.seg[s];
        const float *qr = qres + g.qoff;
        const float sq = warp_eigen_sum(g.dim, [&](int i) { return qr[i]; });
        const float l2 = warp_eigen_sum(g.dim, [&](int i) { return __fmul_rn(qr[i], qr[i]); });
        const int cb0 = g.qoff / 4, ncb = g.dim / 4;
        uint32_t kmin = 0xffffffffu, kmax = 0u;
        for (int k = lane; k < ncb; k += 32) {
            uint32_t a, b;
            codebook_keys(qres + (cb0 + k) * 4, a, b);
            kmin = min(kmin, a);
            kmax = max(kmax, b);
        }
        kmin = __reduce_min_sync(kFull, kmin);
        kmax = __reduce_max_sync(kFull, kmax);
        if (lane == s) {
            sc.sum_q = sq;
            sc.q_l2sqr = l2;
            my_min = kmin;
            my_max = kmax;
        }
    }
    if (lane < ix.S) seg_quant_scalars(my_min, my_max, sc);
    for (int s = 0; s < ix.S; ++s) {
        const SegDev &g = ix.seg[s];
        const float vl = __shfl_sync(kFull, sc.vl, s), delta = __shfl_sync(kFull, sc.delta, s),
                    rd = __shfl_sync(kFull, sc.rdelta, s);
        const int cb0 = g.qoff / 4, ncb = g.dim / 4;
        for (int k = lane; k < ncb; k += 32) quant_codebook(qres + (cb0 + k) * 4, vl, delta, rd, L + (cb0 + k) * 16);
    }
    if (lane < ix.S) {
        seg_epilogue_scalars(ix.seg[lane], prune_all[(size_t)qi * ix.S + lane], sc);
        scal[pair * ix.S + lane] = sc;
    }
}

// The prepared state of cluster c from k_lut's output (lut / scal: this
// pair's), and the residual query, into the CTA's shared memory.
__device__ void load_cluster(const DevIndexView &ix, const float *__restrict__ qrot, const uint16_t *__restrict__ lut,
                             const SegScal *__restrict__ scal, int c, ScanSmem &sm) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const uint4 *src = reinterpret_cast<const uint4 *>(lut);
    uint4 *dst = reinterpret_cast<uint4 *>(sm.lut);
    for (int i = tid; i < ix.Dtot / 2; i += nt) dst[i] = src[i];  // 8 * Dtot bytes
    if (tid < ix.S) sm.scal[tid] = scal[tid];
    for (int s = 0; s < ix.S; ++s) {
        const SegDev &g = ix.seg[s];
        const float *cent = g.cent + (size_t)c * g.dim;
        for (int i = tid; i < g.dim; i += nt) sm.qres[g.qoff + i] = __fsub_rn(qrot[g.qoff + i], cent[i]);
    }
    __syncthreads();
}

// The block's minimum estimate for a pruning stage.  Only its comparisons with
// distk / tau are ever used; without NaN lanes every reduction order gives the
// same minimum (up to the sign of a zero, which no comparison sees), so a
// single key reduction stands in for the reference's min tree.  With a NaN lane
// the tree's order decides the result, and the tree runs.
__device__ __forceinline__ float block_min(float cur) {
    if (!__any_sync(kFull, cur != cur)) return key_to_float(__reduce_min_sync(kFull, fkey(cur)));
    return warp_min_tree(cur);
}

// Pulls cluster c's rotated centroid rows (every segment, 4 * Dtot bytes) into
// L2 ahead of its prepare_cluster: thread tid of nt takes the 128-byte lines
// tid, tid + nt, ... of the rows laid end to end.
__device__ __forceinline__ void prefetch_centroid(const DevIndexView &ix, int c, int tid, int nt) {
    for (int s = 0, first = 0; s < ix.S; ++s) {
        const SegDev &g = ix.seg[s];
        const char *row = reinterpret_cast<const char *>(g.cent + (size_t)c * g.dim);
        const int lines = (4 * g.dim + 127) / 128;
        int l = tid - first;  // first line of this row that is the thread's
        if (l < 0) l += (-l + nt - 1) / nt * nt;
        for (; l < lines; l += nt) asm volatile("prefetch.global.L2 [%0];" ::"l"(row + 128 * l));
        first += lines;
    }
}

// Estimates of one block (this warp, lane = vector).  Fills cd/ipx for every
// segment and, for several segments, the running sum and the pruning-stage
// minima of SAQSearcher::searchCluster steps 1-2 (saq_searcher.hpp:87-132).
// Like the reference, it stops at the first stage whose minimum exceeds the
// bound `tau` (>= every distk the block will meet): such a block has no
// candidate lanes, so the later segments' estimates would never be read.
__device__ void block_estimates(const DevIndexView &ix, int64_t gb, ScanSmem &sm, int w, int lane, float tau) {
    const int S = ix.S;
    if (S == 1) {
        const SegDev &g = ix.seg[0];
        const float on = g.onorm[gb * 32 + lane];
        float ipx = 0.0f, est;
        if (g.bits) est = fast_est(g, sm.lut, sm.scal[0], gb, lane, on, ipx);
        else est = vars_est(sm.scal[0], on);
        sm.cd[w * 32 + lane] = est;
        sm.ipx[w * 32 + lane] = ipx;
        sm.cur[w * 32 + lane] = est;
        return;
    }
    float cur = 0.0f;
    for (int s = 0; s < S; ++s) {
        const float v = vars_est(sm.scal[s], ix.seg[s].onorm[gb * 32 + lane]);
        sm.cd[(w * S + s) * 32 + lane] = v;
        sm.ipx[(w * S + s) * 32 + lane] = 0.0f;
        cur = __fadd_rn(cur, v);
    }
    int k = 0;
    float mi = block_min(cur);
    if (lane == 0) sm.stage[w * (S + 1) + k] = mi;
    ++k;
    for (int s = 0; s < S && !(mi > tau); ++s) {  // mi is warp-uniform
        const SegDev &g = ix.seg[s];
        if (!g.bits) continue;
        const float on = g.onorm[gb * 32 + lane];
        cur = __fsub_rn(cur, sm.cd[(w * S + s) * 32 + lane]);
        float ipx;
        const float f = fast_est(g, sm.lut + 4 * g.qoff, sm.scal[s], gb, lane, on, ipx);
        sm.cd[(w * S + s) * 32 + lane] = f;
        sm.ipx[(w * S + s) * 32 + lane] = ipx;
        cur = __fadd_rn(cur, f);
        mi = block_min(cur);
        if (lane == 0) sm.stage[w * (S + 1) + k] = mi;
        ++k;
    }
    if (lane == 0) sm.nstage[w] = k;
    sm.cur[w * 32 + lane] = cur;
}

// Largest stage minimum (NaN-free ones; NaN when all are NaN or n == 0):
// stages_pass(st, n, tau) == !(stage_max(st, n) > tau).
__device__ __forceinline__ float stage_max(const float *st, int n) {
    float m = __int_as_float(0x7fffffff);
    for (int i = 0; i < n; ++i) m = fmaxf(m, st[i]);
    return m;
}

__device__ __forceinline__ bool stages_pass(const float *st, int n, float tau) {
    for (int i = 0; i < n; ++i)
        if (st[i] > tau) return false;
    return true;
}

// Steps 1-3 of a tile of up to kTileB blocks (warp w <-> blocks t0 + w + k * nwarps
// of the cluster): estimates, candidate masks under `tau`, and the accurate
// distances (multi-segment: accurate - estimate per segment) of every
// candidate lane.  Ends with the partials in sm.part and the masks in sm.cmask.
// The threads [tbase, tbase + nthr) take part (whole warps; a tile then has
// nthr / 32 * kBlocksPerWarp slots); they synchronise on __syncthreads when
// barid is 0, else on the named barrier barid.
__device__ void tile_candidates(const DevIndexView &ix, ScanSmem &sm, int64_t b0, int64_t v0, int nb, int n, int t0,
                                int t_end, float tau, int tbase = 0, int nthr = kScanThreads, int barid = 0) {
    const int S = ix.S, tid = (int)threadIdx.x - tbase, w = tid >> 5, lane = tid & 31;
    const int nwarps = nthr >> 5, nslots = nwarps * kBlocksPerWarp;
    auto sync = [&]() {
        if (barid) asm volatile("bar.sync %0, %1;" ::"r"(barid), "r"(nthr) : "memory");
        else __syncthreads();
    };
#pragma unroll
    for (int k = 0; k < kBlocksPerWarp; ++k) {
        const int slot = w + k * nwarps, b = t0 + slot;
        if (b < t_end) block_estimates(ix, b0 + b, sm, slot, lane, tau);
    }
    // a slot's mask reads only what the same warp's estimates wrote (its cd,
    // cur, stage and nstage rows): a warp barrier orders them
    __syncwarp();
#pragma unroll
    for (int k = 0; k < kBlocksPerWarp; ++k) {
        const int slot = w + k * nwarps, b = t0 + slot;
        if (b < t_end) {
            bool cand;
            if (S == 1) {
                const int cnp = (b == nb - 1) ? (n % 32) : 32;  // scanCluster's last-block count (saq_searcher.hpp:186)
                cand = lane < cnp && sm.cd[slot * 32 + lane] < tau;
            } else {
                cand = stages_pass(sm.stage + slot * (S + 1), sm.nstage[slot], tau) && sm.cur[slot * 32 + lane] < tau &&
                       (b * 32 + lane) < n;
            }
            const uint32_t m = __ballot_sync(kFull, cand);
            if (lane == 0) sm.cmask[slot] = m;
        } else if (lane == 0) {
            sm.cmask[slot] = 0;
        }
    }
    sync();
    // accurate distances: one thread per (candidate vector, segment); the
    // tasks of a segment start on a warp boundary, so a warp's lanes run the
    // same code (one ex-code width and length) instead of diverging over all
    int ncand = 0;
    for (int i = 0; i < nslots; ++i) ncand += __popc(sm.cmask[i]);
    const int P = (ncand + 31) & ~31;
    const int total = S * P;
    auto decode = [&](int r, int &ww, int &j) {
        ww = 0;
        while (r >= __popc(sm.cmask[ww])) {
            r -= __popc(sm.cmask[ww]);
            ++ww;
        }
        uint32_t mk = sm.cmask[ww];
        for (int i = 0; i < r; ++i) mk &= mk - 1;
        j = __ffs(mk) - 1;
    };
    // first pull every task's ex-code row into L1, so the chains below do not
    // wait on memory group by group
    for (int t = tid; t < total; t += nthr) {
        const int s = t / P, r = t - s * P;
        if (r >= ncand) continue;
        int ww, j;
        decode(r, ww, j);
        const SegDev &g = ix.seg[s];
        if (g.bits > 1) {
            const uint8_t *row = g.lcode + (size_t)(v0 + (int64_t)(t0 + ww) * 32 + j) * g.lstride;
            for (int o = 0; o < g.lstride; o += 128) asm volatile("prefetch.global.L1 [%0];" ::"l"(row + o));
        }
    }
    auto finish = [&](int s, int ww, int j, float ex) {
        const int64_t gb = b0 + t0 + ww, gv = v0 + (int64_t)(t0 + ww) * 32 + j;
        const SegDev &g = ix.seg[s];
        const SegScal &sc = sm.scal[s];
        const float acc = accurate_dist(g.onorm[gb * 32 + j], sm.ipx[(ww * S + s) * 32 + j], ex, g.exfac[gv].x, g.bits,
                                        sc.sum_q, sc.q_l2sqr);
        sm.part[(ww * S + s) * 32 + j] = S == 1 ? acc : __fsub_rn(acc, sm.cd[(ww * S + s) * 32 + j]);
    };
    // few tasks: four lanes per task (excode_ip_quad), a quarter of the chain;
    // else one thread per task
    const int P4 = (ncand + 7) & ~7;
    if (S * P4 * 4 <= nthr) {
        // a warp holds 8 tasks of one segment (each segment's tasks padded to a
        // multiple of 8); padding tasks compute on candidate 0 and are discarded
        for (int gl = tid; gl < S * P4 * 4; gl += nthr) {  // warp-uniform: a multiple of 32 lanes
            const int t = gl >> 2, q4 = gl & 3, s = t / P4, r = t - s * P4;
            const bool valid = r < ncand;
            int ww, j;
            decode(valid ? r : 0, ww, j);
            const SegDev &g = ix.seg[s];
            const int64_t gv = v0 + (int64_t)(t0 + ww) * 32 + j;
            const float ex = g.bits > 1 ? excode_ip_quad(sm.qres + g.qoff, g.lcode + (size_t)gv * g.lstride, g.dim,
                                                         g.bits - 1, q4)
                                        : 0.0f;
            if (valid && q4 == 0) finish(s, ww, j, ex);
        }
    } else {
        for (int t = tid; t < total; t += nthr) {
            const int s = t / P, r = t - s * P;
            if (r >= ncand) continue;
            int ww, j;
            decode(r, ww, j);
            const SegDev &g = ix.seg[s];
            const int64_t gv = v0 + (int64_t)(t0 + ww) * 32 + j;
            finish(s, ww, j,
                   g.bits > 1 ? excode_ip_thread(sm.qres + g.qoff, g.lcode + (size_t)gv * g.lstride, g.dim, g.bits - 1)
                              : 0.0f);
        }
    }
    sync();
}

// The reference's sequential decisions for one block (single thread):
// scanCluster's mask-then-insert (saq_searcher.hpp:185-208) or
// searchCluster's stage checks and per-lane partial sums (saq_searcher.hpp:87-160).
// cur: fast estimate (one segment) or running sum; part: [S][32] partials.
__device__ __forceinline__ void replay_block(int S, int n, int nb, int bb, const float *cur, const float *stage,
                                             int nstage, const float *part, uint32_t cm, const uint32_t *ids_v0,
                                             uint32_t *pid, float *pd, int &sz, int topk, float &dk, int *err,
                                             unsigned long long &c_rr) {
    // Only candidate lanes (cm) can pass: every other lane's estimate is >= the
    // tile-start distk >= dk, or lies past the cluster's end.
    (void)n;
    (void)nb;
    (void)err;
    if (S == 1) {
        uint32_t mask = 0;  // scanCluster computes the mask once, at the block's start
        for (uint32_t m = cm; m; m &= m - 1) {
            const int j = __ffs(m) - 1;
            mask |= (uint32_t)(cur[j] < dk) << j;
        }
        while (mask) {
            const int j = __ffs(mask) - 1;
            mask &= mask - 1;
            ++c_rr;
            pool_insert(pid, pd, sz, topk, ids_v0[(int64_t)bb * 32 + j], part[j]);
            dk = sz == topk ? pd[sz - 1] : FLT_MAX;
        }
        return;
    }
    if (!cm || !stages_pass(stage, nstage, dk)) return;
    for (uint32_t m = cm; m; m &= m - 1) {
        const int j = __ffs(m) - 1;
        if (!(cur[j] < dk)) continue;
        ++c_rr;
        float acc = cur[j];
        for (int s = 0; s < S; ++s) {
            acc = __fadd_rn(acc, part[s * 32 + j]);
            if (acc >= dk) break;
        }
        pool_insert(pid, pd, sz, topk, ids_v0[(int64_t)bb * 32 + j], acc);
        dk = sz == topk ? pd[sz - 1] : FLT_MAX;
    }
}

// ResultPool::insert (utils/pool.hpp:17-49) by a whole warp on the pool in
// shared memory: the insert position is the number of entries below `dist`,
// which is what the reference's lower-bound search returns on a sorted pool;
// when `dist` or an entry is NaN (no order) lane 0 runs that search itself.
__device__ __forceinline__ void pool_insert_warp(uint32_t *ids, float *d, int &size, int cap, uint32_t u, float dist) {
    const int lane = threadIdx.x & 31;
    if (size == cap && dist > d[size - 1]) return;
    int lo = 0;
    bool nan = dist != dist;
    for (int i0 = 0; i0 < size; i0 += 32) {
        const int i = i0 + lane;
        const float v = i < size ? d[i] : 0.0f;
        lo += __popc(__ballot_sync(kFull, i < size && v < dist));
        nan = __any_sync(kFull, nan || v != v);
    }
    if (nan) {
        int sz = size;
        if (lane == 0) pool_insert(ids, d, sz, cap, u, dist);
        __syncwarp();
        size = __shfl_sync(kFull, sz, 0);
        return;
    }
    // entries [lo, size) move up one (entry size - 1 lands in the spare slot when full), top chunk first
    for (int i0 = (size >> 5) << 5; i0 >= ((lo + 1) >> 5) << 5; i0 -= 32) {
        const int i = i0 + lane;
        const bool mv = i > lo && i <= size;
        uint32_t pi = 0;
        float pv = 0.0f;
        if (mv) {
            pi = ids[i - 1];
            pv = d[i - 1];
        }
        __syncwarp();
        if (mv) {
            ids[i] = pi;
            d[i] = pv;
        }
        __syncwarp();
    }
    if (lane == 0) {
        ids[lo] = u;
        d[lo] = dist;
    }
    __syncwarp();
    size += size < cap;
}

// The reference's decisions for one block (saq_searcher.hpp:87-160 for several
// segments, scanCluster's mask-then-insert, saq_searcher.hpp:185-208, for one),
// taken by a whole warp.  distk changes only when an insert is accepted, so
// every lane evaluates its own insert under the current distk at once; the
// first accepted lane (in lane order) is inserted, the lanes before it were
// rejected under that same distk, and the lanes after it are evaluated again.
// Rejected inserts thus cost no serial steps.  c_rr counts the lanes whose
// accurate distance the reference computes.
// smax: stage_max of the block's stage minima (several segments).
__device__ __forceinline__ void replay_block_warp(int S, int bb, const float *cur, float smax, const float *part,
                                                  uint32_t cm, const uint32_t *ids_v0, uint32_t *pid, float *pd,
                                                  int &sz, int topk, float &dk, unsigned long long &c_rr) {
    const int lane = threadIdx.x & 31;
    if (!cm) return;
    if (S > 1 && smax > dk) return;
    const bool in = (cm >> lane) & 1u;
    const float c = in ? cur[lane] : FLT_MAX;
    if (S == 1) {
        uint32_t rest = __ballot_sync(kFull, in && c < dk);  // the mask, at the block's start
        c_rr += __popc(rest);
        const float a = in ? part[lane] : FLT_MAX;
        while (rest) {
            const uint32_t ok = rest & __ballot_sync(kFull, !(sz == topk && a > dk));
            if (!ok) break;
            const int j = __ffs(ok) - 1;
            pool_insert_warp(pid, pd, sz, topk, ids_v0[(int64_t)bb * 32 + j], __shfl_sync(kFull, a, j));
            dk = sz == topk ? pd[sz - 1] : FLT_MAX;
            rest &= ~((2u << j) - 1u);
        }
        return;
    }
    uint32_t rest = __ballot_sync(kFull, in);
    while (rest) {
        const uint32_t pass = rest & __ballot_sync(kFull, c < dk);
        float acc = c;
        if ((pass >> lane) & 1u)
            for (int s = 0; s < S; ++s) {
                acc = __fadd_rn(acc, part[s * 32 + lane]);
                if (acc >= dk) break;
            }
        const uint32_t ok = pass & __ballot_sync(kFull, !(sz == topk && acc > dk));
        if (!ok) {
            c_rr += __popc(pass);
            break;
        }
        const int j = __ffs(ok) - 1;
        c_rr += __popc(pass & ((2u << j) - 1u));
        pool_insert_warp(pid, pd, sz, topk, ids_v0[(int64_t)bb * 32 + j], __shfl_sync(kFull, acc, j));
        dk = sz == topk ? pd[sz - 1] : FLT_MAX;
        rest &= ~((2u << j) - 1u);
    }
}

// The reference's decisions for the nblk (<= 32) blocks of a tile, in order, by
// one warp: lane i first reads block i's candidate mask and (several segments)
// the largest of its stage minima, and a ballot keeps the blocks that can
// change the pool under the distk at the tile's start.  distk only decreases,
// so a block dropped here (no candidate lane, or a stage minimum above distk)
// would be skipped by replay_block_warp as well; the rest are replayed in order.
// Returns the tile's candidate lanes (for the tally).
__device__ __forceinline__ unsigned replay_tile_warp(int S, int t0, int nblk, const ScanSmem &v, const uint32_t *ids_v0,
                                                     uint32_t *pid, float *pd, int &sz, int topk, float &dk,
                                                     unsigned long long &c_rr) {
    const int lane = threadIdx.x & 31;
    uint32_t cm = 0;
    float smax = 0.0f;
    if (lane < nblk) {
        cm = v.cmask[lane];
        if (S > 1 && cm) smax = stage_max(v.stage + lane * (S + 1), v.nstage[lane]);
    }
    uint32_t live = __ballot_sync(kFull, cm != 0 && !(S > 1 && smax > dk));
    while (live) {
        const int ww = __ffs(live) - 1;
        live &= live - 1;
        replay_block_warp(S, t0 + ww, v.cur + ww * 32, __shfl_sync(kFull, smax, ww),
                          S == 1 ? v.part + ww * 32 : v.part + ww * S * 32, __shfl_sync(kFull, cm, ww), ids_v0, pid, pd,
                          sz, topk, dk, c_rr);
    }
    return __reduce_add_sync(kFull, __popc(cm));
}

struct ScanTally {
    unsigned long long blocks = 0, vecs = 0, rr = 0, spec = 0;
};

// Exact sequential scan of probes [p_begin, p_end) of one query, continuing
// the pool held in shared memory (pool_size / distk in shared memory).  Each
// nonempty probed cluster's LUT comes from the batched preparation when `lut`
// is set (this query's pairs: probe p's at lut + p * 4 * Dtot, scal + p * S),
// else it is built here.
__device__ void scan_probes(const DevIndexView &ix, const uint32_t *__restrict__ probe, int p_begin, int p_end,
                            const float *__restrict__ qrot, const float *__restrict__ prune, int topk, ScanSmem &sm,
                            int &pool_size, float &distk, ScanTally &tl, const uint16_t *__restrict__ lut,
                            const SegScal *__restrict__ scal) {
    const int S = ix.S, tid = threadIdx.x;
    for (int p = p_begin; p < p_end; ++p) {
        const int c = (int)probe[p];
        const int64_t b0 = ix.blk_off[c], v0 = ix.vec_off[c];
        const int nb = (int)(ix.blk_off[c + 1] - b0), n = (int)(ix.vec_off[c + 1] - v0);
        tl.blocks += nb;
        tl.vecs += n;
        if (nb == 0) continue;
        if (lut) load_cluster(ix, qrot, lut + (size_t)p * 4 * ix.Dtot, scal + (size_t)p * S, c, sm);
        else prepare_cluster(ix, qrot, prune, c, sm);
        if (p + 1 < p_end) prefetch_centroid(ix, (int)probe[p + 1], tid, blockDim.x);
        for (int t0 = 0; t0 < nb; t0 += kTileB) {
            tile_candidates(ix, sm, b0, v0, nb, n, t0, nb, distk);
            if (tid < 32) {
                float dk = distk;
                int sz = pool_size;
                const unsigned nc = replay_tile_warp(S, t0, min(kTileB, nb - t0), sm, ix.ids + v0, sm.pool_id, sm.pool_d,
                                                     sz, topk, dk, tl.rr);
                if (tid == 0) {
                    tl.spec += nc;
                    distk = dk;
                    pool_size = sz;
                }
            }
            __syncthreads();
        }
    }
}

__device__ void init_pool(ScanSmem &sm, int topk, int &pool_size, float &distk) {
    for (int i = threadIdx.x; i <= topk; i += blockDim.x) {
        sm.pool_id[i] = 0;
        sm.pool_d[i] = 0.0f;
    }
    if (threadIdx.x == 0) {
        pool_size = 0;
        distk = FLT_MAX;
    }
    __syncthreads();
}

__device__ void flush_tally(const ScanTally &tl, unsigned long long *counters) {
    if (threadIdx.x == 0 && counters) {
        atomicAdd(counters + 0, tl.blocks);
        atomicAdd(counters + 1, tl.vecs);
        atomicAdd(counters + 2, tl.rr);
        atomicAdd(counters + 3, tl.spec);
    }
}

// The pool as the reference returns it (unfilled slots id 0), then, for a
// row longer than this query's k, id 0 / FLT_MAX up to k_max.
__device__ void write_results(const ScanSmem &sm, int pool_size, int topk, int k_max, uint32_t *out_ids, float *out_d) {
    for (int i = threadIdx.x; i < k_max; i += blockDim.x) {
        out_ids[i] = i < topk ? sm.pool_id[i] : 0u;
        if (out_d) out_d[i] = i < pool_size && i < topk ? sm.pool_d[i] : FLT_MAX;
    }
}

// ------------------------------------------------------------------ warp-specialised scan
// k_scan with the replay overlapped: warp 0 replays tile t (the reference's
// decisions, the pool, distk) while warps 1-7 compute the estimates, masks and
// accurate distances of tile t + 1 into the other of two tile buffers.  The
// workers' bound for a tile is the distk the replay had published when the tile
// began, which is at least every distk the tile will meet in the replay (distk
// only shrinks), so the candidate lanes remain a superset and the answers are
// k_scan's.  Named barriers: 1 among the workers (224 threads); 2 + b "tile in
// buffer b written" (workers arrive, warp 0 waits); 4 + b "buffer b replayed"
// (warp 0 arrives, the workers wait before they overwrite it).
constexpr int kWsWorkers = kScanThreads - 32;
constexpr int kWsSlots = (kWsWorkers / 32) * kBlocksPerWarp;  // blocks per tile

struct WsTile {
    int64_t v0;  // first vector of the tile's cluster
    int t0;      // first block of the tile within the cluster
};

__host__ __device__ inline size_t ws_tile_bytes(int S) {
    return 3 * align16(sizeof(float) * kTileB * S * 32) + align16(sizeof(float) * kTileB * 32) +
           align16(sizeof(float) * kTileB * (S + 1)) + align16(sizeof(uint32_t) * kTileB) +
           align16(sizeof(int) * kTileB);
}

__host__ __device__ inline size_t ws_smem_bytes(int Dtot, int S, int topk, int xstride) {
    return scan_smem_bytes(Dtot, S, topk, xstride) + ws_tile_bytes(S);
}

// The tile buffer `b` of a warp-specialised layout: buffer 0 is the base
// layout's, buffer 1 the arrays appended at `extra`.
__device__ __forceinline__ ScanSmem ws_view(const ScanSmem &sm, char *extra, int S, int b) {
    if (!b) return sm;
    ScanSmem v = sm;
    size_t o = 0;
    v.cd = (float *)(extra + o);
    o += align16(sizeof(float) * kTileB * S * 32);
    v.ipx = (float *)(extra + o);
    o += align16(sizeof(float) * kTileB * S * 32);
    v.part = (float *)(extra + o);
    o += align16(sizeof(float) * kTileB * S * 32);
    v.cur = (float *)(extra + o);
    o += align16(sizeof(float) * kTileB * 32);
    v.stage = (float *)(extra + o);
    o += align16(sizeof(float) * kTileB * (S + 1));
    v.cmask = (uint32_t *)(extra + o);
    o += align16(sizeof(uint32_t) * kTileB);
    v.nstage = (int *)(extra + o);
    return v;
}

__device__ __forceinline__ void named_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void named_arrive(int id, int n) {
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}

__global__ void __launch_bounds__(kScanThreads, kScanMinCtas) k_scan_ws(DevIndexView ix, const uint32_t *__restrict__ probe,
                                                          QueryShape qsh, const float *__restrict__ qrot_all,
                                                          const float *__restrict__ prune_all,
                                                          uint32_t *__restrict__ out_ids, float *__restrict__ out_d,
                                                          unsigned long long *__restrict__ counters, int xstride,
                                                          const uint8_t *__restrict__ deferred,
                                                          const int *__restrict__ order) {
    extern __shared__ __align__(16) char smem_raw[];
    const int qi = order ? order[blockIdx.x] : (int)blockIdx.x;
    if (deferred && deferred[qi]) return;  // answered by the split pass
    const int np = qsh.np_of(qi), topk = qsh.k_of(qi), S = ix.S, tid = threadIdx.x;
    ScanSmem sm = scan_smem_layout(smem_raw, ix.Dtot, S, qsh.k_max, xstride);
    char *extra = smem_raw + scan_smem_bytes(ix.Dtot, S, qsh.k_max, xstride);
    __shared__ WsTile meta[2];
    __shared__ int pool_size;
    __shared__ float distk;
    volatile float *vdistk = &distk;
    init_pool(sm, topk, pool_size, distk);
    const uint32_t *pr = probe + (size_t)qi * qsh.np_max;
    const float *qrot = qrot_all + (size_t)qi * ix.Dtot, *prune = prune_all + (size_t)qi * ix.S;
    int ntiles = 0;
    if (tid >= 32) {
        // ---- workers: LUTs, estimates, masks, accurate distances
        unsigned long long blocks = 0, vecs = 0;
        for (int p = 0; p < np; ++p) {
            const int c = (int)pr[p];
            const int64_t b0 = ix.blk_off[c], v0 = ix.vec_off[c];
            const int nb = (int)(ix.blk_off[c + 1] - b0), n = (int)(ix.vec_off[c + 1] - v0);
            blocks += nb;
            vecs += n;
            if (nb == 0) continue;
            prepare_cluster(ix, qrot, prune, c, sm, 32, 1);
            for (int t0 = 0; t0 < nb; t0 += kWsSlots, ++ntiles) {
                const int b = ntiles & 1;
                if (ntiles >= 2) named_sync(4 + b, kScanThreads);  // the replay of tile ntiles - 2 is done
                ScanSmem v = ws_view(sm, extra, S, b);
                if (tid == 32) meta[b] = WsTile{v0, t0};
                const float tau = __shfl_sync(kFull, *vdistk, 0);  // warp-uniform, as block_estimates wants
                tile_candidates(ix, v, b0, v0, nb, n, t0, min(nb, t0 + kWsSlots), tau, 32, kWsWorkers, 1);
                __threadfence_block();
                named_arrive(2 + b, kScanThreads);
            }
        }
        for (int t = max(0, ntiles - 2); t < ntiles; ++t) named_sync(4 + (t & 1), kScanThreads);  // the last replays
        if (tid == 32 && counters) {
            atomicAdd(counters + 0, blocks);
            atomicAdd(counters + 1, vecs);
        }
    } else {
        // ---- warp 0: the reference's decisions, in order
        unsigned long long rr = 0, spec = 0;
        float dk = distk;
        int sz = pool_size;
        for (int p = 0; p < np; ++p) {
            const int c = (int)pr[p];
            const int nb = (int)(ix.blk_off[c + 1] - ix.blk_off[c]);
            for (int t0 = 0; t0 < nb; t0 += kWsSlots, ++ntiles) {
                const int b = ntiles & 1;
                named_sync(2 + b, kScanThreads);  // tile ntiles written
                const ScanSmem v = ws_view(sm, extra, S, b);
                const WsTile mt = meta[b];
                const unsigned nc = replay_tile_warp(S, mt.t0, min(kWsSlots, nb - mt.t0), v, ix.ids + mt.v0,
                                                     sm.pool_id, sm.pool_d, sz, topk, dk, rr);
                if (tid == 0) {
                    spec += nc;
                    *vdistk = dk;
                    pool_size = sz;
                }
                __threadfence_block();
                __syncwarp();
                named_arrive(4 + b, kScanThreads);  // buffer b may be overwritten
            }
        }
        if (tid == 0 && counters) {
            atomicAdd(counters + 2, rr);
            atomicAdd(counters + 3, spec);
        }
    }
    __syncthreads();
    write_results(sm, pool_size, topk, qsh.k_max, out_ids + (size_t)qi * qsh.k_max,
                  out_d ? out_d + (size_t)qi * qsh.k_max : nullptr);
}

// ------------------------------------------------------------------ warp scan
// Throughput form for batches: one WARP per query, no CTA barriers.  The warp
// walks its probes and blocks in the reference's order with the exact current
// distk (no speculation): lane v estimates vector v of the block, the lanes
// that pass re-rank themselves (thread-level chains, all segments), and lane 0
// applies the reference's insert sequence.  Each warp owns its LUTs and pool
// in shared memory.
constexpr int kWarpsPerCta = 4;

struct WarpSmem {
    uint16_t *lut;   // 4 * Dtot
    float *qres;     // Dtot
    SegScal *scal;   // S
    float *cd, *ipx, *part;  // S * 32 each
    float *cur;      // 32
    float *stage;    // S + 1
    uint32_t *pool_id;
    float *pool_d;   // topk + 1 each
};

__host__ __device__ inline size_t warp_smem_bytes(int Dtot, int S, int topk) {
    return align16(2 * 4 * (size_t)Dtot) + align16(4 * (size_t)Dtot) + align16(sizeof(SegScal) * S) +
           3 * align16(4 * 32 * (size_t)S) + align16(4 * 32) + align16(4 * (size_t)(S + 1)) +
           2 * align16(4 * (size_t)(topk + 1));
}

__device__ WarpSmem warp_smem_layout(char *base, int Dtot, int S, int topk) {
    WarpSmem w;
    size_t o = 0;
    w.lut = (uint16_t *)(base + o);
    o += align16(2 * 4 * (size_t)Dtot);
    w.qres = (float *)(base + o);
    o += align16(4 * (size_t)Dtot);
    w.scal = (SegScal *)(base + o);
    o += align16(sizeof(SegScal) * S);
    w.cd = (float *)(base + o);
    o += align16(4 * 32 * (size_t)S);
    w.ipx = (float *)(base + o);
    o += align16(4 * 32 * (size_t)S);
    w.part = (float *)(base + o);
    o += align16(4 * 32 * (size_t)S);
    w.cur = (float *)(base + o);
    o += align16(4 * 32);
    w.stage = (float *)(base + o);
    o += align16(4 * (size_t)(S + 1));
    w.pool_id = (uint32_t *)(base + o);
    o += align16(4 * (size_t)(topk + 1));
    w.pool_d = (float *)(base + o);
    return w;
}

// Lut::prepare for every segment of cluster c, by one warp.
__device__ void prepare_cluster_warp(const DevIndexView &ix, const float *__restrict__ qrot,
                                     const float *__restrict__ prune, int c, WarpSmem &ws) {
    const int lane = threadIdx.x & 31, S = ix.S;
    for (int i = lane; i < ix.Dtot; i += 32) {
        int s = 0;
        while (s + 1 < S && i >= ix.seg[s + 1].qoff) ++s;
        const SegDev &g = ix.seg[s];
        ws.qres[i] = __fsub_rn(qrot[i], g.cent[(size_t)c * g.dim + (i - g.qoff)]);
    }
    __syncwarp();
    for (int s = 0; s < S; ++s) {
        const SegDev &g = ix.seg[s];
        const float *qr = ws.qres + g.qoff;
        const float sum_q = warp_eigen_sum(g.dim, [&](int i) { return qr[i]; });
        const float q2 = warp_eigen_sum(g.dim, [&](int i) { return __fmul_rn(qr[i], qr[i]); });
        const int ncb = g.dim / 4;
        float lo = FLT_MAX, hi = -FLT_MAX;
        for (int cb = lane; cb < ncb; cb += 32) {
            float t[16];
            lut_entries(qr + cb * 4, t);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                lo = fminf(lo, t[j]);
                hi = fmaxf(hi, t[j]);
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(kFull, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(kFull, hi, o));
        }
        const float delta = (float)__ddiv_rn((double)__fsub_rn(hi, lo), 65536.0 - 0.01);
        uint16_t *lut = ws.lut + 4 * g.qoff;
        for (int cb = lane; cb < ncb; cb += 32) {
            float t[16];
            lut_entries(qr + cb * 4, t);
            uint32_t packed[8];
#pragma unroll
            for (int j = 0; j < 16; j += 2) {
                const uint32_t a = (uint16_t)(int)__fdiv_rn(__fsub_rn(t[j], lo), delta);
                const uint32_t b = (uint16_t)(int)__fdiv_rn(__fsub_rn(t[j + 1], lo), delta);
                packed[j / 2] = a | (b << 16);
            }
            uint4 *dst = reinterpret_cast<uint4 *>(lut + cb * 16);
            dst[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
            dst[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
        }
        if (lane == 0) {
            SegScal &sc = ws.scal[s];
            sc.delta = delta;
            sc.vl = lo;
            sc.sum_vl = (float)__dmul_rn(__dadd_rn((double)lo, __dmul_rn(0.5, (double)delta)), (double)(float)ncb);
            sc.sum_q = sum_q;
            sc.q_l2sqr = q2;
            sc.q_l2norm = sqrtf(q2);
            sc.c1 = (float)__dsub_rn(__dmul_rn(0.5, (double)sum_q), (double)__fmul_rn(0.58f, sc.q_l2norm));
            const float one_over_sqrtD = (float)__ddiv_rn(1.0, (double)sqrtf((float)g.dim));
            sc.c2 = __fmul_rn(__fdiv_rn(4.0f, 0.8f), one_over_sqrtD);
            sc.vfac = __fsub_rn(q2, __fmul_rn(2.0f, prune[s]));
        }
    }
    __syncwarp();
}

__global__ void __launch_bounds__(kWarpsPerCta * 32) k_scan_warp(DevIndexView ix, const uint32_t *__restrict__ probe,
                                                                 int nprobe, int nq, const float *__restrict__ qrot_all,
                                                                 const float *__restrict__ prune_all, int topk,
                                                                 uint32_t *__restrict__ out_ids,
                                                                 float *__restrict__ out_d,
                                                                 unsigned long long *__restrict__ counters,
                                                                 size_t per_warp) {
    extern __shared__ __align__(16) char smem_raw[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, S = ix.S;
    const int qi = blockIdx.x * kWarpsPerCta + w;
    if (qi >= nq) return;
    WarpSmem ws = warp_smem_layout(smem_raw + w * per_warp, ix.Dtot, S, topk);
    for (int i = lane; i <= topk; i += 32) {
        ws.pool_id[i] = 0;
        ws.pool_d[i] = 0.0f;
    }
    int sz = 0;
    float dk = FLT_MAX;
    unsigned long long c_blocks = 0, c_vecs = 0, c_rr = 0, c_spec = 0;
    const uint32_t *pr = probe + (size_t)qi * nprobe;
    const float *qrot = qrot_all + (size_t)qi * ix.Dtot, *prune = prune_all + (size_t)qi * S;
    for (int p = 0; p < nprobe; ++p) {
        const int c = (int)pr[p];
        prepare_cluster_warp(ix, qrot, prune, c, ws);
        const int64_t b0 = ix.blk_off[c], v0 = ix.vec_off[c];
        const int nb = (int)(ix.blk_off[c + 1] - b0), n = (int)(ix.vec_off[c + 1] - v0);
        c_blocks += nb;
        c_vecs += n;
        for (int b = 0; b < nb; ++b) {
            const int64_t gb = b0 + b;
            // estimates (saq_searcher.hpp:87-132 / 185-195), lane = vector
            float cur = 0.0f;
            int nst = 0;
            bool pass = true;
            if (S == 1) {
                const SegDev &g = ix.seg[0];
                const float on = g.onorm[gb * 32 + lane];
                float ipx = 0.0f;
                const float est = g.bits ? fast_est(g, ws.lut, ws.scal[0], gb, lane, on, ipx) : vars_est(ws.scal[0], on);
                ws.cd[lane] = est;
                ws.ipx[lane] = ipx;
                cur = est;
            } else {
                float cdv[kMaxSeg];
                for (int s = 0; s < S; ++s) {
                    cdv[s] = vars_est(ws.scal[s], ix.seg[s].onorm[gb * 32 + lane]);
                    cur = __fadd_rn(cur, cdv[s]);
                }
                float mi = warp_min_tree(cur);
                pass = !(mi > dk);
                ws.stage[0] = mi;  // all lanes write the same value
                nst = 1;
                for (int s = 0; s < S && pass; ++s) {
                    const SegDev &g = ix.seg[s];
                    if (!g.bits) continue;
                    const float on = g.onorm[gb * 32 + lane];
                    cur = __fsub_rn(cur, cdv[s]);
                    float ipx;
                    cdv[s] = fast_est(g, ws.lut + 4 * g.qoff, ws.scal[s], gb, lane, on, ipx);
                    ws.ipx[s * 32 + lane] = ipx;
                    cur = __fadd_rn(cur, cdv[s]);
                    mi = warp_min_tree(cur);
                    pass = !(mi > dk);
                    ++nst;
                }
                for (int s = 0; s < S; ++s) ws.cd[s * 32 + lane] = cdv[s];
            }
            // candidates under the exact distk at the block's start
            bool cand;
            if (S == 1) {
                const int cnp = (b == nb - 1) ? (n % 32) : 32;  // scanCluster's last-block count
                cand = lane < cnp && cur < dk;
            } else {
                cand = pass && cur < dk && (b * 32 + lane) < n;
            }
            const uint32_t cm = __ballot_sync(kFull, cand);
            if (!cm) continue;
            if (cand) {  // re-rank this lane's vector: every segment, thread-level chains
                const int64_t gv = v0 + (int64_t)b * 32 + lane;
                for (int s = 0; s < S; ++s) {
                    const SegDev &g = ix.seg[s];
                    const float ex = g.bits > 1 ? excode_ip_thread(ws.qres + g.qoff, g.lcode + (size_t)gv * g.lstride,
                                                                   g.dim, g.bits - 1)
                                                : 0.0f;
                    const float acc = accurate_dist(g.onorm[gb * 32 + lane], ws.ipx[s * 32 + lane], ex, g.exfac[gv].x,
                                                    g.bits, ws.scal[s].sum_q, ws.scal[s].q_l2sqr);
                    ws.part[s * 32 + lane] = S == 1 ? acc : __fsub_rn(acc, ws.cd[s * 32 + lane]);
                }
            }
            ws.cur[lane] = cur;
            __syncwarp();
            if (lane == 0) {
                c_spec += __popc(cm);
                replay_block(S, n, nb, b, ws.cur, ws.stage, 0, ws.part, cm, ix.ids + v0, ws.pool_id, ws.pool_d, sz,
                             topk, dk, nullptr, c_rr);
            }
            dk = __shfl_sync(kFull, dk, 0);
            sz = __shfl_sync(kFull, sz, 0);
            __syncwarp();
        }
    }
    if (lane == 0 && counters) {
        atomicAdd(counters + 0, c_blocks);
        atomicAdd(counters + 1, c_vecs);
        atomicAdd(counters + 2, c_rr);
        atomicAdd(counters + 3, c_spec);
    }
    __syncwarp();
    for (int i = lane; i < topk; i += 32) {
        out_ids[(size_t)qi * topk + i] = ws.pool_id[i];
        if (out_d) out_d[(size_t)qi * topk + i] = i < sz ? ws.pool_d[i] : FLT_MAX;
    }
}

// ------------------------------------------------------------------ split scan
// For latency-bound calls (one query, or a few).  The first tile of the
// nearest cluster is scanned exactly; the pool's distk afterwards, tau1, bounds
// distk for the rest of the scan (distk never grows).  Every remaining (probe,
// tile) is processed in parallel across the GPU under tau1; each block with a
// lane below tau1 leaves a record in a slot indexed by its position in scan
// order.  A final pass per query walks the positions in order and replays the
// reference's decisions on the records.  Blocks without a record cannot insert
// anything (none of their lanes is below tau1 >= distk), so the replay is exact.
constexpr int kTileBlocks = 16;
constexpr int kSpecChunk = 8;          // speculative tiles per work chunk of k_scan_spec
constexpr int kSpecChunkPrepared = 2;  // ... when the LUTs come from the batched preparation
constexpr int kFirstBlocks = 16;  // exact prefix of a deferred query (its distk bounds the first level)
// Levels of the speculation for deferred queries, in tiles after the split
// point: [0, 8), [8, 64), [64, end) by default; the autotuner may pick another
// set (each level's replay leaves the exact pool whose distk bounds the next
// level's speculation: more levels, tighter bounds, more launches).
constexpr int kMaxSpecLevels = 5;
constexpr int kSpecLevelSets[][kMaxSpecLevels] = {
    {0, 8, 64, -1, -1},
    {0, 4, 32, 256, -1},
    {0, 16, 128, -1, -1},
    {0, 8, 64, 512, -1},
    {0, 64, -1, -1, -1},
};
constexpr int kNumSpecLevelSets = (int)(sizeof(kSpecLevelSets) / sizeof(kSpecLevelSets[0]));
constexpr int kDeferBlocks = 1024;  // a query scanning more blocks than this takes the split pass
                                     // (SAQG_DEFER_BLOCKS overrides it; 0 disables deferral)

struct SplitState {
    int *nlist;          // number of queries on the list (device)
    int *work_next;      // next chunk of the level's speculative tiles (reset by k_tile_prefix)
    int *qlist;          // [cap] slot -> query id
    int cap;             // slots
    uint32_t *pool_id;   // [cap][topk]
    float *pool_d;       // [cap][topk]
    int *pool_size;      // [cap]
    float *tau;          // [cap]
    int *tile_off;       // [cap][nprobe + 1] tiles before probe p
    int *blk_base;       // [cap][nprobe] scan-order position of the probe's first block
    int *split_p;        // [cap] probe where the speculative part starts (nprobe: none)
    int *split_b;        // [cap] block of that probe's cluster where it starts
    int *q_tile_off;     // [cap + 1]
    int *npos;           // [cap] scan positions (blocks) of the query
    int64_t *pos_off;    // [cap] first record position reserved for the slot
    unsigned long long *pos_used;  // record positions handed out so far
    // [pos_cap] per record (NaN: none): x the smallest candidate estimate, y the
    // largest stage minimum, z the smallest value a candidate lane's accept test
    // can see (its accurate distance; several segments: every running sum),
    // -inf when one of them is NaN
    float4 *summ;
    float *rec;          // [pos_cap][rec_words]
    int64_t pos_cap;
    int rec_words;
    QueryShape qsh;      // per-query nprobe and k (strides np_max, k_max)
    int first_blocks;    // exact prefix: at least this many blocks, and a full pool
    // the level being speculated and replayed: tiles [t_lo, t_hi) after the split
    // point of each query (distk at the level's start bounds its speculation)
    int t_lo, t_hi;
    int final_level;     // the last level writes the results, the others the pool
};

// Scan-order position of the first block of tile t after a query's split
// point (npos when t is past its last tile).
__device__ __forceinline__ int tile_pos(const SplitState &st, int slot, int t) {
    const int npm = st.qsh.np_max;
    const int *to = st.tile_off + (size_t)slot * (npm + 1);
    if (t >= to[npm]) return st.npos[slot];
    int lo = 0, hi = npm;  // probe: last p with to[p] <= t
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (to[mid] <= t) lo = mid;
        else hi = mid;
    }
    const int first = lo == st.split_p[slot] ? st.split_b[slot] : 0;
    return st.blk_base[(size_t)slot * npm + lo] + first + (t - to[lo]) * kTileBlocks;
}

__host__ __device__ inline int rec_words_of(int S) { return (8 + (S + 1) + 32 + 32 * S + 3) & ~3; }

__device__ __forceinline__ int list_len(const SplitState &st) { return min(*st.nlist, st.cap); }

__global__ void __launch_bounds__(kScanThreads, kScanMinCtas) k_scan_first(DevIndexView ix, const uint32_t *__restrict__ probe,
                                                             const float *__restrict__ qrot_all,
                                                             const float *__restrict__ prune_all, SplitState st, int *__restrict__ err,
                                                             unsigned long long *__restrict__ counters, int xstride,
                                                             Prepared prep) {
    extern __shared__ __align__(16) char smem_raw[];
    const int S = ix.S, tid = threadIdx.x;
    // slots round-robin over a grid sized to the machine (the list length is known on the device only)
    for (int slot = blockIdx.x; slot < list_len(st); slot += gridDim.x) {
        const int qi = st.qlist[slot];
        const int np_max = st.qsh.np_max, k_max = st.qsh.k_max;
        const int nprobe = st.qsh.np_of(qi), topk = st.qsh.k_of(qi);
        ScanSmem sm = scan_smem_layout(smem_raw, ix.Dtot, S, k_max, xstride);
        __shared__ int pool_size;
        __shared__ float distk;
        ScanTally tl;
        init_pool(sm, topk, pool_size, distk);
        const uint32_t *pr = probe + (size_t)qi * np_max;
        const float *qrot = qrot_all + (size_t)qi * ix.Dtot, *prune = prune_all + (size_t)qi * S;
        // the exact prefix, as scan_probes does: whole tiles in scan order until at
        // least kFirstBlocks blocks are done and the pool is full (its distk then
        // bounds every later distk, so it can serve as the speculation bound)
        int sp_p = nprobe, sp_b = 0;
        for (int p = 0; p < nprobe && sp_p == nprobe; ++p) {
            const int c = (int)pr[p];
            const int64_t b0 = ix.blk_off[c], v0 = ix.vec_off[c];
            const int nb = (int)(ix.blk_off[c + 1] - b0), n = (int)(ix.vec_off[c + 1] - v0);
            bool prepared = false;
            for (int t0 = 0; t0 < nb; t0 += kTileB) {
                if (tl.blocks >= st.first_blocks && pool_size == topk) {
                    sp_p = p;
                    sp_b = t0;
                    break;
                }
                if (!prepared) {
                    if (prep.has(slot)) load_cluster(ix, qrot, prep.lut_of(slot, p, ix.Dtot), prep.scal_of(slot, p, S), c, sm);
                    else prepare_cluster(ix, qrot, prune, c, sm);
                    prepared = true;
                }
                const int te = min(nb, t0 + kTileB);
                tl.blocks += te - t0;
                tl.vecs += min(n, te * 32) - t0 * 32;
                tile_candidates(ix, sm, b0, v0, nb, n, t0, nb, distk);
                if (tid < 32) {
                    float dk = distk;
                    int sz = pool_size;
                    const unsigned nc = replay_tile_warp(S, t0, te - t0, sm, ix.ids + v0, sm.pool_id, sm.pool_d, sz, topk, dk,
                                                         tl.rr);
                    if (tid == 0) {
                        tl.spec += nc;
                        distk = dk;
                        pool_size = sz;
                    }
                }
                __syncthreads();
            }
        }
        flush_tally(tl, counters);
        for (int i = tid; i < topk; i += blockDim.x) {
            st.pool_id[(size_t)slot * k_max + i] = sm.pool_id[i];
            st.pool_d[(size_t)slot * k_max + i] = sm.pool_d[i];
        }
        if (tid == 0) {
            st.pool_size[slot] = pool_size;
            st.tau[slot] = distk;
            st.split_p[slot] = sp_p;
            st.split_b[slot] = sp_b;
            int tiles = 0;
            int64_t pos = 0;
            for (int p = 0; p < nprobe; ++p) {
                const int c = (int)pr[p];
                const int nb = (int)(ix.blk_off[c + 1] - ix.blk_off[c]);
                st.tile_off[(size_t)slot * (np_max + 1) + p] = tiles;
                st.blk_base[(size_t)slot * np_max + p] = (int)pos;
                const int rest = p < sp_p ? 0 : p == sp_p ? nb - sp_b : nb;
                tiles += (rest + kTileBlocks - 1) / kTileBlocks;
                pos += nb;
            }
            for (int p = nprobe; p <= np_max; ++p) st.tile_off[(size_t)slot * (np_max + 1) + p] = tiles;
            if (pos != st.npos[slot]) *err = 2;
        }
        __syncthreads();  // the next slot reuses the shared state
    }
}

// Work offsets of the level's tiles: slot q holds tiles [t_lo, t_hi) of its own.
// One CTA of kPrefixThreads: each thread sums a contiguous run of slots, a
// block-wide exclusive scan of the run sums, then each run is written.
constexpr int kPrefixThreads = 256;
__global__ void __launch_bounds__(kPrefixThreads) k_tile_prefix(SplitState st) {
    __shared__ int wsum[kPrefixThreads / 32];
    const int nprobe = st.qsh.np_max, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int n = list_len(st);
    const int per = (n + kPrefixThreads - 1) / kPrefixThreads, q0 = min(n, tid * per), q1 = min(n, q0 + per);
    auto count = [&](int q) {
        const int nt = st.tile_off[(size_t)q * (nprobe + 1) + nprobe];
        return max(0, min(nt, st.t_hi) - min(nt, st.t_lo));
    };
    int run = 0;
    for (int q = q0; q < q1; ++q) run += count(q);
    int x = run;  // inclusive scan within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    constexpr int kW = kPrefixThreads / 32;
    if (w == 0) {
        int v = lane < kW ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        if (lane < kW) wsum[lane] = v;  // inclusive over warps
    }
    __syncthreads();
    int acc = x - run + (w ? wsum[w - 1] : 0);
    for (int q = q0; q < q1; ++q) {
        st.q_tile_off[q] = acc;
        acc += count(q);
    }
    if (tid == kPrefixThreads - 1) {
        st.q_tile_off[n] = wsum[kPrefixThreads / 32 - 1];
        *st.work_next = 0;
    }
}

__global__ void __launch_bounds__(kScanThreads, kScanMinCtas) k_scan_spec(DevIndexView ix, const uint32_t *__restrict__ probe,
                                                            int nprobe, const float *__restrict__ qrot_all,
                                                            const float *__restrict__ prune_all, SplitState st,
                                                            unsigned long long *__restrict__ counters, int xstride,
                                                            Prepared prep) {
    extern __shared__ __align__(16) char smem_raw[];
    const int S = ix.S, tid = threadIdx.x;
    ScanSmem sm = scan_smem_layout(smem_raw, ix.Dtot, S, 1, xstride);
    ScanTally tl;
    const int nl = list_len(st);
    const int total = st.q_tile_off[nl];
    // chunks of consecutive tiles (mostly of one cluster: one LUT) taken from a
    // shared counter: tiles differ widely in cost (candidates, pruning stages),
    // so equal shares per CTA leave a long tail.  When every listed query has
    // prepared LUTs a cluster switch is a copy, and chunks are short.
    // at least about four chunks per CTA, so that a small level (few queries)
    // still spreads over the whole grid
    const bool all_prepared = prep.lut && prep.slots >= nl;
    const int ct = max(1, min(all_prepared ? kSpecChunkPrepared : kSpecChunk, total / (4 * (int)gridDim.x)));
    __shared__ int chunk;
    int last_slot = -1, last_c = -1;
    for (;;) {
        if (tid == 0) chunk = atomicAdd(st.work_next, 1);
        __syncthreads();
        const int w_begin = chunk * ct, w_end = min(total, w_begin + ct);
        __syncthreads();  // every thread has read `chunk` before thread 0 takes the next
        if (w_begin >= total) break;
        for (int wi = w_begin; wi < w_end; ++wi) {
            int lo = 0, hi = nl;  // slot: last with q_tile_off[slot] <= wi
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (st.q_tile_off[mid] <= wi) lo = mid;
                else hi = mid;
            }
            const int slot = lo, q = st.qlist[slot];
            const int local = st.t_lo + (wi - st.q_tile_off[slot]);
            const int *to = st.tile_off + (size_t)slot * (nprobe + 1);
            int plo = 0, phi = nprobe;  // probe: last p with to[p] <= local
            while (phi - plo > 1) {
                const int mid = (plo + phi) >> 1;
                if (to[mid] <= local) plo = mid;
                else phi = mid;
            }
            const int p = plo, tile = local - to[p];
            const int c = (int)probe[(size_t)q * nprobe + p];
            if (slot != last_slot || c != last_c) {  // LUTs survive across tiles of one cluster
                if (prep.has(slot)) load_cluster(ix, qrot_all + (size_t)q * ix.Dtot, prep.lut_of(slot, p, ix.Dtot),
                                                 prep.scal_of(slot, p, S), c, sm);
                else prepare_cluster(ix, qrot_all + (size_t)q * ix.Dtot, prune_all + (size_t)q * S, c, sm);
                last_slot = slot;
                last_c = c;
            }
            const int64_t b0 = ix.blk_off[c], v0 = ix.vec_off[c];
            const int nb = (int)(ix.blk_off[c + 1] - b0), n = (int)(ix.vec_off[c + 1] - v0);
            const int first = p == st.split_p[slot] ? st.split_b[slot] : 0;
            const int bstart = first + tile * kTileBlocks, bend = min(nb, bstart + kTileBlocks);
            if (tid == 0) {
                tl.blocks += bend - bstart;
                tl.vecs += min(n, bend * 32) - bstart * 32;
            }
            const float tau = st.tau[slot];
            const int64_t base = st.blk_base[(size_t)slot * nprobe + p];
            for (int t0 = bstart; t0 < bend; t0 += kTileB) {
                tile_candidates(ix, sm, b0, v0, nb, n, t0, bend, tau);
                const int lane = tid & 31;
                for (int k = 0; k < kBlocksPerWarp; ++k) {
                    const int w = (tid >> 5) + k * kScanWarps, b = t0 + w;
                    if (b < bend) {
                        const uint32_t cm = sm.cmask[w];
                        const int64_t pos = base + b;
                        if (cm && pos < st.npos[slot]) {
                            float *r = st.rec + (size_t)(st.pos_off[slot] + pos) * st.rec_words;
                            uint32_t *ri = reinterpret_cast<uint32_t *>(r);
                            // summary: a later distk below the minimum estimate, or below a stage minimum,
                            // leaves the block without effect
                            const bool in = (cm >> lane) & 1u;
                            float mn = in ? sm.cur[w * 32 + lane] : __int_as_float(0x7fffffff);
                            float mx = (S > 1 && lane < sm.nstage[w]) ? sm.stage[w * (S + 1) + lane] : __int_as_float(0x7fffffff);
                            // ... and a later distk below every value the lane's accept test can
                            // compare (replay_block_warp: the accurate distance, or each running sum)
                            float mz = __int_as_float(0x7f800000);
                            if (in) {
                                if (S == 1) {
                                    mz = sm.part[w * 32 + lane];
                                } else {
                                    float acc = sm.cur[w * 32 + lane];
                                    for (int s2 = 0; s2 < S; ++s2) {
                                        acc = __fadd_rn(acc, sm.part[(w * S + s2) * 32 + lane]);
                                        mz = fminf(mz, acc);
                                        if (acc != acc) mz = -__int_as_float(0x7f800000);
                                    }
                                }
                                if (mz != mz) mz = -__int_as_float(0x7f800000);
                            }
    #pragma unroll
                            for (int o = 16; o; o >>= 1) {
                                mn = fminf(mn, __shfl_xor_sync(kFull, mn, o));
                                mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
                                mz = fminf(mz, __shfl_xor_sync(kFull, mz, o));
                            }
                            if (lane == 0) {
                                ri[0] = (uint32_t)pos;
                                ri[1] = cm;
                                ri[2] = (uint32_t)(S == 1 ? 0 : sm.nstage[w]);
                                ri[3] = (uint32_t)c;
                                ri[4] = (uint32_t)b;
                                ri[5] = (uint32_t)(uint64_t)v0;
                                ri[6] = (uint32_t)((uint64_t)v0 >> 32);
                                ri[7] = __float_as_uint(mx);
                                st.summ[st.pos_off[slot] + pos] = make_float4(mn, mx, mz, 0.0f);
                                if (counters) atomicAdd(counters + 3, (unsigned long long)__popc(cm));
                            }
                            if (S > 1 && lane <= S) r[8 + lane] = sm.stage[w * (S + 1) + lane];
                            r[8 + (S + 1) + lane] = sm.cur[w * 32 + lane];
                            for (int s = 0; s < S; ++s)
                                r[8 + (S + 1) + 32 + s * 32 + lane] = sm.part[(w * S + s) * 32 + lane];
                        }
                    }
                }
                __syncthreads();
            }
        }
    }
    if (tid == 0 && counters) {
        atomicAdd(counters + 0, tl.blocks);
        atomicAdd(counters + 1, tl.vecs);
    }
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Whether a staged record changes the pool under the current distk / pool
// size (some lane's insert would be accepted), and how many of its lanes the
// reference evaluates accurately when nothing earlier in the record changes
// distk.  Warp-uniform.
__device__ __forceinline__ bool record_effect(int S, const float *rec, float dk, int sz, int topk, int &count) {
    const int lane = threadIdx.x & 31;
    const uint32_t *ri = reinterpret_cast<const uint32_t *>(rec);
    const uint32_t cm = ri[1];
    count = 0;
    if (!cm || (S > 1 && __uint_as_float(ri[7]) > dk)) return false;
    const float *cur = rec + 8 + (S + 1), *part = cur + 32;
    const bool in = (cm >> lane) & 1u;
    const float c = in ? cur[lane] : FLT_MAX;
    const bool pass = in && c < dk;
    count = __popc(__ballot_sync(kFull, pass));
    float acc = c;
    if (S == 1) {
        acc = pass ? part[lane] : FLT_MAX;
    } else if (pass) {
        for (int s = 0; s < S; ++s) {
            acc = __fadd_rn(acc, part[s * 32 + lane]);
            if (acc >= dk) break;
        }
    }
    return __any_sync(kFull, pass && !(sz == topk && acc > dk));
}

constexpr int kReplayRecs = 32;  // records per staged chunk (double-buffered)
constexpr int kReplayPer = 4;    // scan positions per thread in a window

// Per query on the list: walk its scan positions in order, kScanThreads at a
// time.  A record can matter only if a candidate estimate lies below distk and
// no stage minimum above it; distk only shrinks, so positions whose summary
// fails the distk at the window's start are dropped at once.  The rest are
// staged into shared memory by asynchronous copies, kReplayRecs at a time
// (the next chunk in flight while the current one is evaluated).  In a chunk,
// every warp evaluates records under the current distk; the first record with
// an accepted insert is replayed exactly by warp 0 (the records before it
// change nothing and only add their counts), and evaluation resumes after it.
__global__ void __launch_bounds__(kScanThreads) k_scan_replay(DevIndexView ix, SplitState st,
                                                              uint32_t *__restrict__ out_ids, float *__restrict__ out_d,
                                                              unsigned long long *__restrict__ counters, int xstride) {
    extern __shared__ __align__(16) char smem_raw[];
    const int S = ix.S;
    // slots round-robin over a grid sized to the machine (the list length is known on the device only)
    for (int slot = blockIdx.x; slot < list_len(st); slot += gridDim.x) {
        const int qi = st.qlist[slot];
        const int k_max = st.qsh.k_max, topk = st.qsh.k_of(qi);
        ScanSmem sm = scan_smem_layout(smem_raw, ix.Dtot, S, k_max, xstride);
        float *stage_buf = reinterpret_cast<float *>(smem_raw + scan_smem_bytes(ix.Dtot, S, k_max, xstride));
        __shared__ int pool_size;
        __shared__ float distk;
        __shared__ int list[kScanThreads * kReplayPer];
        __shared__ int warp_cnt[kScanWarps];
        __shared__ int eff[kReplayRecs], cnt[kReplayRecs];
        __shared__ int s_next, s_plo, s_phi;
        __shared__ int eff_pos[kReplayRecs], n_eff;  // records replayed in the current chunk
        __shared__ float eff_dk[kReplayRecs], c_dk0;
        const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
        for (int i = tid; i < topk; i += blockDim.x) {
            sm.pool_id[i] = st.pool_id[(size_t)slot * k_max + i];
            sm.pool_d[i] = st.pool_d[(size_t)slot * k_max + i];
        }
        if (tid == 0) {
            pool_size = st.pool_size[slot];
            distk = st.tau[slot];
            s_plo = tile_pos(st, slot, st.t_lo);  // this level's scan positions
            s_phi = tile_pos(st, slot, st.t_hi);
        }
        const int np = st.npos[slot];
        const float4 *su = st.summ + st.pos_off[slot];
        const float *rq = st.rec + (size_t)st.pos_off[slot] * st.rec_words;
        const int RW = st.rec_words, R16 = RW / 4;
        unsigned long long rr = 0;
        __syncthreads();
        const int pos_end = min(np, s_phi);
        for (int base = s_plo; base < pos_end; base += kScanThreads * kReplayPer) {
            // thread t tests positions base + kReplayPer t .. + kReplayPer - 1; a
            // block-wide prefix of the counts keeps the list in position order
            const int p0 = base + kReplayPer * tid;
            const float dk0 = distk;
            // with a full pool a lane is accepted only at a value <= distk: a record whose
            // every such value exceeds distk (summary z) changes nothing and is not staged.
            // With counters kept, the lanes the reference evaluates in such a record are
            // counted after each chunk under the distk at its position (count_dropped).
            const bool zf = pool_size == topk;
            const int wend = min(pos_end, base + kScanThreads * kReplayPer);
            bool f[kReplayPer];
            int mine = 0;
    #pragma unroll
            for (int r = 0; r < kReplayPer; ++r) {
                f[r] = false;
                if (p0 + r < pos_end) {
                    const float4 v = su[p0 + r];
                    f[r] = v.x < dk0 && !(v.y > dk0) && !(zf && v.z > dk0);
                }
                mine += f[r];
            }
            int incl = mine;
    #pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(kFull, incl, o);
                if (lane >= o) incl += v;
            }
            if (lane == 31) warp_cnt[w] = incl;
            __syncthreads();
            int off = incl - mine, total = 0;
            for (int i = 0; i < kScanWarps; ++i) {
                if (i < w) off += warp_cnt[i];
                total += warp_cnt[i];
            }
    #pragma unroll
            for (int r = 0; r < kReplayPer; ++r)
                if (f[r]) list[off++] = p0 + r;
            __syncthreads();
            const int nch = (total + kReplayRecs - 1) / kReplayRecs;
            // lanes with candidate estimate below the distk at their position in the
            // records of [lo, hi) that the accept bound dropped (distk: c_dk0, then after
            // each of the n_eff records replayed in this range, in position order)
            auto count_dropped = [&](int lo, int hi) {
                unsigned long long add = 0;
                for (int p = lo + tid; p < hi; p += kScanThreads) {
                    const float4 v = su[p];
                    if (!(v.x < dk0 && !(v.y > dk0) && v.z > dk0)) continue;
                    float dkp = c_dk0;
                    for (int e = 0; e < n_eff; ++e)
                        if (eff_pos[e] < p) dkp = eff_dk[e];
                    if (S > 1 && v.y > dkp) continue;  // a stage minimum above distk: no lane evaluated
                    const float *rec = rq + (size_t)p * RW;
                    const float *cur = rec + 8 + (S + 1);
                    for (uint32_t m = reinterpret_cast<const uint32_t *>(rec)[1]; m; m &= m - 1)
                        add += cur[__ffs(m) - 1] < dkp;
                }
                if (add) atomicAdd(counters + 2, add);
            };
            if (nch == 0 && counters && zf) {
                if (tid == 0) {
                    c_dk0 = dk0;
                    n_eff = 0;
                }
                __syncthreads();
                count_dropped(base, wend);
                __syncthreads();
            }
            auto issue = [&](int k) {
                const int c0 = k * kReplayRecs, cn = min(kReplayRecs, total - c0);
                float *buf = stage_buf + (size_t)(k & 1) * kReplayRecs * RW;
                for (int i = tid; i < cn * R16; i += kScanThreads) {
                    const int r = i / R16, e = i - r * R16;
                    cp_async16(buf + (size_t)r * RW + 4 * e, rq + (size_t)list[c0 + r] * RW + 4 * e);
                }
                cp_async_commit();
            };
            if (nch) issue(0);
            for (int k = 0; k < nch; ++k) {
                if (k + 1 < nch) {
                    issue(k + 1);
                    cp_async_wait<1>();
                } else {
                    cp_async_wait<0>();
                }
                __syncthreads();
                const float *buf = stage_buf + (size_t)(k & 1) * kReplayRecs * RW;
                const int c0 = k * kReplayRecs, cn = min(kReplayRecs, total - c0);
                if (tid == 0) {  // read by warp 0 (thread 0 first) and, after the chunk, by count_dropped
                    c_dk0 = distk;
                    n_eff = 0;
                }
                int r0 = 0;
                while (r0 < cn) {
                    const float dk = distk;
                    const int sz = pool_size;
                    for (int r = r0 + w; r < cn; r += kScanWarps) {
                        int c;
                        const bool e = record_effect(S, buf + (size_t)r * RW, dk, sz, topk, c);
                        if (lane == 0) {
                            eff[r] = e;
                            cnt[r] = c;
                        }
                    }
                    __syncthreads();
                    if (w == 0) {
                        const bool mine = lane >= r0 && lane < cn;
                        const uint32_t hit = __ballot_sync(kFull, mine && eff[lane]);
                        const int rs = hit ? __ffs(hit) - 1 : cn;  // first record that changes the pool
                        int c = (lane >= r0 && lane < rs) ? cnt[lane] : 0;
                        for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(kFull, c, o);
                        rr += (unsigned long long)c;
                        if (rs < cn) {
                            const float *rec = buf + (size_t)rs * RW;
                            const uint32_t *ri = reinterpret_cast<const uint32_t *>(rec);
                            const int64_t v0 = (int64_t)(((uint64_t)ri[6] << 32) | ri[5]);
                            float dkw = dk;
                            int szw = sz;
                            replay_block_warp(S, (int)ri[4], rec + 8 + (S + 1), __uint_as_float(ri[7]),
                                              rec + 8 + (S + 1) + 32, ri[1], ix.ids + v0, sm.pool_id, sm.pool_d, szw, topk,
                                              dkw, rr);
                            if (lane == 0) {
                                distk = dkw;
                                pool_size = szw;
                                eff_pos[n_eff] = list[c0 + rs];
                                eff_dk[n_eff] = dkw;
                                ++n_eff;
                            }
                        }
                        if (lane == 0) s_next = rs + 1;
                    }
                    __syncthreads();
                    r0 = s_next;
                }
                if (counters && zf) {
                    count_dropped(k == 0 ? base : list[c0 - 1] + 1, k + 1 == nch ? wend : list[c0 + cn - 1] + 1);
                    __syncthreads();
                }
            }
        }
        __syncthreads();
        if (tid == 0 && counters) atomicAdd(counters + 2, rr);
        if (st.final_level) {
            write_results(sm, pool_size, topk, k_max, out_ids + (size_t)qi * k_max,
                          out_d ? out_d + (size_t)qi * k_max : nullptr);
        } else {  // the pool and its distk carry over to the next level
            for (int i = tid; i < topk; i += blockDim.x) {
                st.pool_id[(size_t)slot * k_max + i] = sm.pool_id[i];
                st.pool_d[(size_t)slot * k_max + i] = sm.pool_d[i];
            }
            if (tid == 0) {
                st.pool_size[slot] = pool_size;
                st.tau[slot] = distk;
            }
        }
        __syncthreads();  // the next slot reuses the shared state
    }
}

// One CTA per query: the whole probe list sequentially (queries deferred to
// the split pass are skipped).
__global__ void __launch_bounds__(kScanThreads, kScanMinCtas) k_scan(DevIndexView ix, const uint32_t *__restrict__ probe,
                                                       QueryShape qsh, const float *__restrict__ qrot_all,
                                                       const float *__restrict__ prune_all,
                                                       uint32_t *__restrict__ out_ids, float *__restrict__ out_d,
                                                       unsigned long long *__restrict__ counters, int xstride,
                                                       const uint8_t *__restrict__ deferred,
                                                       const int *__restrict__ order, Prepared prep) {
    extern __shared__ __align__(16) char smem_raw[];
    const int qi = order ? order[blockIdx.x] : (int)blockIdx.x;
    if (deferred && deferred[qi]) return;  // answered by the split pass
    const int np = qsh.np_of(qi), topk = qsh.k_of(qi);
    ScanSmem sm = scan_smem_layout(smem_raw, ix.Dtot, ix.S, qsh.k_max, xstride);
    __shared__ int pool_size;
    __shared__ float distk;
    ScanTally tl;
    init_pool(sm, topk, pool_size, distk);
    scan_probes(ix, probe + (size_t)qi * qsh.np_max, 0, np, qrot_all + (size_t)qi * ix.Dtot,
                prune_all + (size_t)qi * ix.S, topk, sm, pool_size, distk, tl,
                prep.has(qi) ? prep.lut_of(qi, 0, ix.Dtot) : nullptr, prep.has(qi) ? prep.scal_of(qi, 0, ix.S) : nullptr);
    flush_tally(tl, counters);
    write_results(sm, pool_size, topk, qsh.k_max, out_ids + (size_t)qi * qsh.k_max,
                  out_d ? out_d + (size_t)qi * qsh.k_max : nullptr);
}

// Launch order of the CTA scan, heaviest queries first (blocks of their probes,
// in power-of-two classes; the order inside a class is arbitrary), so that a
// long query does not start in the last wave; the split pass's queries (deferred)
// last, as their CTAs only return.  One CTA of kOrderThreads.
constexpr int kOrderThreads = 1024;
constexpr int kOrderMinQueries = 1024;  // batches from which the CTA scan is launched heaviest first
__global__ void __launch_bounds__(kOrderThreads) k_order(DevIndexView ix, const uint32_t *__restrict__ probe, QueryShape qsh,
                                                         int nq, const int *__restrict__ qblocks,
                                                         const uint8_t *__restrict__ deferred,
                                                         int *__restrict__ order) {
    __shared__ int cnt[33], cur[33];
    const int tid = threadIdx.x;
    if (tid < 33) cnt[tid] = 0;
    __syncthreads();
    auto cls = [&](int qi) {
        if (deferred && deferred[qi]) return 32;
        int64_t total = 0;
        if (qblocks) {
            total = qblocks[qi];
        } else {
            const int np = qsh.np_of(qi);
            for (int p = 0; p < np; ++p) {
                const int c = (int)probe[(size_t)qi * qsh.np_max + p];
                total += ix.blk_off[c + 1] - ix.blk_off[c];
            }
        }
        return 31 - min(31, 63 - __clzll((long long)total + 1));  // heavier: smaller class
    };
    for (int qi = tid; qi < nq; qi += kOrderThreads) atomicAdd(&cnt[cls(qi)], 1);
    __syncthreads();
    if (tid == 0) {
        int acc = 0;
        for (int k = 0; k < 33; ++k) {
            cur[k] = acc;
            acc += cnt[k];
        }
    }
    __syncthreads();
    for (int qi = tid; qi < nq; qi += kOrderThreads) order[atomicAdd(&cur[cls(qi)], 1)] = qi;
}

// Puts the queries whose probes hold more than `defer_blocks` blocks (giant Zipf
// clusters; every query when defer_blocks < 0) on the split list, each with
// record positions for all its blocks, heaviest first while the record space
// lasts: queries in power-of-two classes of their blocks, heavy classes first,
// in query order inside a class.  What does not fit is left to the CTA scan,
// which then holds the lighter queries.  Writes every query's block count
// (qblocks: the CTA scan's launch order) unless k_qblocks has (have_qblocks).
// One CTA of up to kDeferThreads (a multiple of 32); thread t owns the queries
// [t * per, (t + 1) * per).
constexpr int kDeferThreads = 1024;
constexpr int kQblocksMinQueries = 256;  // from this batch size the block counts come from k_qblocks

// Blocks of each query's probes, one thread per query (k_defer's input for
// large batches, where its single CTA would sum them serially).
__global__ void k_qblocks(DevIndexView ix, const uint32_t *__restrict__ probe, QueryShape qsh, int nq,
                          int *__restrict__ qblocks) {
    const int qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    int64_t total = 0;
    const int np = qsh.np_of(qi);
    for (int p = 0; p < np; ++p) {
        const int c = (int)probe[(size_t)qi * qsh.np_max + p];
        total += ix.blk_off[c + 1] - ix.blk_off[c];
    }
    qblocks[qi] = total < (int64_t)INT_MAX ? (int)total : INT_MAX;
}

__global__ void __launch_bounds__(kDeferThreads) k_defer(DevIndexView ix, const uint32_t *__restrict__ probe, int nq,
                                                         int defer_blocks, SplitState st, int *__restrict__ qblocks,
                                                         int have_qblocks, uint8_t *__restrict__ deferred) {
    __shared__ long long wsum_b[kDeferThreads / 32];
    __shared__ int wsum_n[kDeferThreads / 32], hist[32];
    __shared__ long long s_base;  // record positions handed out
    __shared__ int s_slot;        // list entries handed out
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nt = blockDim.x, nw = nt >> 5;
    const int per = (nq + nt - 1) / nt, q0 = min(nq, tid * per), q1 = min(nq, q0 + per);
    if (!have_qblocks)
        for (int qi = q0; qi < q1; ++qi) {
            int64_t total = 0;
            const int np = st.qsh.np_of(qi);
            for (int p = 0; p < np; ++p) {
                const int c = (int)probe[(size_t)qi * st.qsh.np_max + p];
                total += ix.blk_off[c + 1] - ix.blk_off[c];
            }
            qblocks[qi] = total < (int64_t)INT_MAX ? (int)total : INT_MAX;  // read back by this thread only
        }
    auto eligible = [&](int qi) {
        return defer_blocks < 0 || (defer_blocks > 0 && qblocks[qi] > defer_blocks);
    };
    auto cls = [&](int qi) { return 31 - min(31, 31 - __clz(qblocks[qi] + 1)); };  // heavier: smaller class
    if (tid < 32) hist[tid] = 0;
    if (tid == 0) {
        s_base = 0;
        s_slot = 0;
    }
    __syncthreads();
    for (int qi = q0; qi < q1; ++qi) {
        deferred[qi] = 0;
        if (eligible(qi)) atomicAdd(&hist[cls(qi)], 1);
    }
    __syncthreads();
    for (int c = 0; c < 32; ++c) {
        if (hist[c] == 0) continue;  // uniform: read after a barrier
        long long mine = 0;
        int cnt = 0;
        for (int qi = q0; qi < q1; ++qi)
            if (eligible(qi) && cls(qi) == c) {
                mine += qblocks[qi];
                ++cnt;
            }
        // exclusive prefix of (blocks, count) over the threads, in thread order
        long long xb = mine;
        int xn = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long yb = __shfl_up_sync(0xffffffffu, xb, o);
            const int yn = __shfl_up_sync(0xffffffffu, xn, o);
            if (lane >= o) {
                xb += yb;
                xn += yn;
            }
        }
        if (lane == 31) {
            wsum_b[w] = xb;
            wsum_n[w] = xn;
        }
        __syncthreads();
        long long before_b = xb - mine;
        int before_n = xn - cnt;
        for (int i = 0; i < w; ++i) {  // the warps before this one
            before_b += wsum_b[i];
            before_n += wsum_n[i];
        }
        const long long base = s_base;
        const int slot0 = s_slot;
        __syncthreads();  // every thread has read s_base / s_slot and the warp sums
        // the accepted queries of the class are a prefix of its order: positions grow along it
        long long acc_b = 0;
        int acc_n = 0;
        long long pos = base + before_b;
        int k = before_n;
        for (int qi = q0; qi < q1; ++qi) {
            if (!eligible(qi) || cls(qi) != c) continue;
            const int t = qblocks[qi];
            if (pos + t > st.pos_cap) break;
            const int slot = slot0 + k;
            st.qlist[slot] = qi;
            st.pos_off[slot] = pos;
            st.npos[slot] = t;
            deferred[qi] = 1;
            pos += t;
            ++k;
            acc_b += t;
            ++acc_n;
        }
        // the class's accepted blocks and queries
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            acc_b += __shfl_xor_sync(0xffffffffu, acc_b, o);
            acc_n += __shfl_xor_sync(0xffffffffu, acc_n, o);
        }
        if (lane == 0) {
            wsum_b[w] = acc_b;
            wsum_n[w] = acc_n;
        }
        __syncthreads();
        if (tid == 0) {
            for (int i = 0; i < nw; ++i) {
                s_base += wsum_b[i];
                s_slot += wsum_n[i];
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        *st.nlist = s_slot;
        *st.pos_used = (unsigned long long)s_base;
    }
}

// ------------------------------------------------------------------ estimate
// IVF::estimate: every vector of the probed clusters (no pruning); one CTA per
// probed cluster, outputs at the cluster's offset in probe order.
__global__ void __launch_bounds__(kScanThreads) k_estimate(DevIndexView ix, const uint32_t *__restrict__ probe,
                                                           const int64_t *__restrict__ out_off,
                                                           const float *__restrict__ qrot,
                                                           const float *__restrict__ prune, uint32_t *__restrict__ o_ids,
                                                           float *__restrict__ o_acc, float *__restrict__ o_fast,
                                                           float *__restrict__ o_vars, int xstride) {
    extern __shared__ __align__(16) char smem_raw[];
    const int S = ix.S;
    ScanSmem sm = scan_smem_layout(smem_raw, ix.Dtot, S, 1, xstride);
    const int p = blockIdx.x, c = (int)probe[p];
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    prepare_cluster(ix, qrot, prune, c, sm);
    const int64_t b0 = ix.blk_off[c], v0 = ix.vec_off[c];
    const int nb = (int)(ix.blk_off[c + 1] - b0), n = (int)(ix.vec_off[c + 1] - v0);
    const int64_t base = out_off[p];
    for (int b = w; b < nb; b += kScanWarps) {
        const int64_t gb = b0 + b;
        float fsum = 0.0f, vsum = 0.0f;
        for (int s = 0; s < S; ++s) {
            const SegDev &g = ix.seg[s];
            const float on = g.onorm[gb * 32 + lane];
            const float v = vars_est(sm.scal[s], on);
            float ipx = 0.0f;
            const float f = g.bits ? fast_est(g, sm.lut + 4 * g.qoff, sm.scal[s], gb, lane, on, ipx) : v;
            sm.ipx[(w * S + s) * 32 + lane] = ipx;
            fsum = __fadd_rn(fsum, f);
            vsum = __fadd_rn(vsum, v);
        }
        __syncwarp();
        const int nv = min(32, n - b * 32);
        if (lane < nv) {  // one thread per vector, all segments in order
            const int64_t gv = v0 + (int64_t)b * 32 + lane;
            float acc = 0.0f;
            for (int s = 0; s < S; ++s) {
                const SegDev &g = ix.seg[s];
                const float ex = g.bits > 1 ? excode_ip_thread(sm.qres + g.qoff, g.lcode + (size_t)gv * g.lstride,
                                                               g.dim, g.bits - 1)
                                            : 0.0f;
                acc = __fadd_rn(acc, accurate_dist(g.onorm[gb * 32 + lane], sm.ipx[(w * S + s) * 32 + lane], ex,
                                                   g.exfac[gv].x, g.bits, sm.scal[s].sum_q, sm.scal[s].q_l2sqr));
            }
            const int64_t o = base + (int64_t)b * 32 + lane;
            o_ids[o] = ix.ids[gv];
            o_acc[o] = acc;
            o_fast[o] = fsum;
            o_vars[o] = vsum;
        }
        __syncwarp();
    }
}

struct Bump {
    char *base;
    size_t off = 0;
    template <class T>
    T *take(size_t count) {
        off = align16(off);
        T *p = reinterpret_cast<T *>(base + off);
        off += sizeof(T) * count;
        return p;
    }
};

// List entries of the split pass that get the batched preparation: as many as
// kPrepCap holds (nprobe pairs each), at most nq; 0 below kPrepMinQueries
// queries, where the scan CTAs build each cluster's state in the shorter latency
// (256 threads per LUT).  12 GB holds every query of a 4,096-query batch at
// nprobe 256 with D = 1024 (8.8 GB; the CTA scan's copy is as large again), a
// few percent of the device beside the index.
constexpr size_t kPrepCap = (size_t)12 << 30;
constexpr int64_t kPrepMinQueries = 64;
size_t prep_pair_bytes(const Index &I) { return 8 * (size_t)I.view.Dtot + sizeof(SegScal) * I.view.S; }
int64_t prep_slots(const Index &I, int64_t nq, int64_t nprobe) {
    if (nq < kPrepMinQueries) return 0;
    return std::min<int64_t>(nq, (int64_t)(kPrepCap / (prep_pair_bytes(I) * (size_t)nprobe)));
}
size_t prep_bytes(const Index &I, int64_t nq, int64_t nprobe) {
    const size_t pairs = (size_t)prep_slots(I, nq, nprobe) * nprobe;
    return pairs ? align16(pairs * 8 * (size_t)I.view.Dtot) + align16(pairs * sizeof(SegScal) * I.view.S) : 0;
}

size_t search_scratch_bytes(const Index &I, int64_t nq, int64_t topk, int64_t nprobe, bool host_io) {
    size_t b = 0;
    auto add = [&](size_t x) { b += align16(x); };
    add(4 * (size_t)nq * I.D);                 // queries (host io)
    add(4 * (size_t)nq * I.K);                 // centroid distances
    add(8 * (size_t)nq * I.K);                 // exact-select work (fallback)
    add(4 * (size_t)nq * nprobe);              // probe ids
    add(4 * (size_t)nq * I.view.Dtot);         // rotated queries
    add(4 * (size_t)nq * I.view.S);            // prune bounds
    add(2 * (size_t)nq * I.D);                 // BF16 queries (probe GEMM)
    add((size_t)nq);                           // shortlist: queries on the full exact path
    add(4 * (size_t)nq);                       // ... and their list
    add(4 * (size_t)nq);                       // CTA scan launch order
    add(4 * (size_t)nq * topk * 2);            // outputs (host io)
    add(4 * (size_t)nq * 2);                   // per-query nprobe / k
    add(64);                                   // flags
    add(64);                                   // counters
    add(prep_bytes(I, nq, nprobe));            // prepared LUTs of the split list
    if (prep_slots(I, nq, nprobe) == nq) add(prep_bytes(I, nq, nprobe));  // ... and of the CTA scan's queries
    (void)host_io;
    return b + 256;
}

size_t split_scratch_bytes(const Index &I, int64_t cap, int64_t topk, int64_t nprobe, int64_t pos_cap) {
    size_t b = 0;
    auto add = [&](size_t x) { b += align16(x); };
    add(4 * 16);                                 // nlist, pos_used, work_next
    add(4 * (size_t)cap);                        // qlist
    add(4 * (size_t)cap * topk);
    add(4 * (size_t)cap * topk);
    add(4 * (size_t)cap);
    add(4 * (size_t)cap);
    add(4 * (size_t)cap * (nprobe + 1));
    add(4 * (size_t)cap * nprobe);
    add(8 * (size_t)cap);                        // split_p, split_b
    add(4 * (size_t)(cap + 1));
    add(4 * (size_t)cap);                        // npos
    add(8 * (size_t)cap);                        // pos_off
    add(16 * (size_t)pos_cap);                   // record summaries
    add(4 * (size_t)pos_cap * rec_words_of(I.view.S));
    add((size_t)cap);                            // deferred flags, one per query
    add(4 * (size_t)cap);                        // blocks of each query's probes
    return b + 256;
}

// Record positions of the split pass for a batch: every block of every query
// (`want`), bounded by scratch memory.
int64_t split_positions(const Index &I, int64_t want) {
    const size_t per = 4 * (size_t)rec_words_of(I.view.S) + 16;
    size_t budget = (size_t)8 << 30;
    if (const char *e = std::getenv("SAQG_SPLIT_RECORD_BYTES"))  // tests: a small budget forces the overflow path
        budget = std::max<size_t>(per, (size_t)std::atoll(e));
    const int64_t by_mem = (int64_t)(budget / per);
    return std::max<int64_t>(1, std::min(want, by_mem));
}

// Which exact scan serves a call: the split scan for latency-bound calls (few
// queries), one CTA per query for batches, unless the tuned shape says
// otherwise.  SAQG_SCAN_MODE=seq|split|warp forces one (tests).
// 0: one CTA per query, 1: split scan, 2: one warp per query.
int scan_mode(int64_t nq, int64_t topk, const ScanTune &t) {
    const char *m = std::getenv("SAQG_SCAN_MODE");
    if (m && std::string(m) == "seq") return 0;
    if (m && std::string(m) == "split") return 1;
    if (m && std::string(m) == "warp") return topk <= 256 ? 2 : 0;
    if (m && std::string(m) == "ws") return 0;
    if (t.mode == 0 || t.mode == 1) return t.mode;
    if (t.mode == 3) return 0;
    if (t.mode == 2) return topk <= 256 ? 2 : 0;
    if (nq <= 16) return 1;
    return 0;
}

// Whether mode 0's CTA scan runs warp-specialised (scan mode 3).
bool scan_ws(const ScanTune &t) {
    if (const char *m = std::getenv("SAQG_SCAN_MODE")) return std::string(m) == "ws";
    return t.mode == 3;
}

// The deferral threshold of mode 0 (blocks of a query's probes above which it
// takes the split pass; 0: never).
int defer_threshold(const ScanTune &t) {
    int defer = t.defer_blocks >= 0 ? t.defer_blocks : kDeferBlocks;
    if (const char *e = std::getenv("SAQG_DEFER_BLOCKS")) defer = std::max(0, std::atoi(e));
    return defer;
}

// Whether no query of a mode-0 call can be deferred: its nprobe largest
// clusters hold no more blocks than the threshold.
bool no_deferral(const Index &I, int64_t nprobe, const ScanTune &t) {
    const int defer = defer_threshold(t);
    return defer == 0 || I.max_blocks_of_probes(nprobe) <= defer;
}

// Per-query nprobe / k copies clamped to the call's maxima (graph launches read
// caller-written device arrays; an out-of-range value must not index past a row).
__global__ void k_clamp_shape(const int *__restrict__ np, const int *__restrict__ k, int nq, int np_max, int k_max,
                              int *__restrict__ np_out, int *__restrict__ k_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    if (np) np_out[i] = min(max(np[i], 1), np_max);
    if (k) k_out[i] = min(max(k[i], 1), k_max);
}

int xstride_of(const DevIndexView &) { return 0; }  // re-rank reads ex-codes in place (no staging buffer)

void check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error{SAQG_ERR_CUDA, std::string(what) + " launch failed: " + cudaGetErrorString(e)};
}

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) once per (kernel, device)
// and size: a call's host time matters for single queries.
void ensure_smem(const void *fn, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, size_t> have;
    int dev = 0;
    SAQG_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    size_t &h = have[{fn, dev}];
    if (bytes <= h) return;
    SAQG_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    h = bytes;
}

// The CTA-per-query scan of `nq` queries (deferred ones skipped): k_scan, with
// the batched LUTs that prep_of(deferred) launches and returns (or none), or its
// warp-specialised form k_scan_ws, which gives the same answers.
void launch_cta_scan(bool ws, const DevIndexView &ix, const uint32_t *probe, const QueryShape &qsh, const float *qrot,
                     const float *prune, uint32_t *ids, float *d, unsigned long long *cnt, int xs,
                     const uint8_t *deferred, int64_t nq, int *order, const int *qblocks,
                     const std::function<Prepared(const uint8_t *)> &prep_of, cudaStream_t st) {
    if (order) {
        k_order<<<1, kOrderThreads, 0, st>>>(ix, probe, qsh, (int)nq, qblocks, deferred, order);
        check_launch("k_order");
    }
    if (ws) {
        const size_t smem = ws_smem_bytes(ix.Dtot, ix.S, qsh.k_max, xs);
        SAQG_REQUIRE(smem <= 220 * 1024, "dimension / topk too large for the scan kernel's shared memory");
        ensure_smem((const void *)k_scan_ws, smem);
        k_scan_ws<<<(unsigned)nq, kScanThreads, smem, st>>>(ix, probe, qsh, qrot, prune, ids, d, cnt, xs, deferred,
                                                             order);
        check_launch("k_scan_ws");
        return;
    }
    const size_t smem = scan_smem_bytes(ix.Dtot, ix.S, qsh.k_max, xs);
    SAQG_REQUIRE(smem <= 200 * 1024, "dimension / topk too large for the scan kernel's shared memory");
    ensure_smem((const void *)k_scan, smem);
    const Prepared prep = prep_of(deferred);
    k_scan<<<(unsigned)nq, kScanThreads, smem, st>>>(ix, probe, qsh, qrot, prune, ids, d, cnt, xs, deferred, order,
                                                      prep);
    check_launch("k_scan");
}

// SMs x resident CTAs of a kernel (per device and shared-memory size), cached.
// Streaming multiprocessors of the current device, cached.
int sm_count() {
    static std::mutex mu;
    static std::map<int, int> have;
    int dev = 0;
    SAQG_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    auto it = have.find(dev);
    if (it != have.end()) return it->second;
    int sms = 0;
    SAQG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    return have[dev] = std::max(1, sms);
}

int full_grid(const void *fn, int threads, size_t smem) {
    static std::mutex mu;
    static std::map<std::tuple<const void *, int, size_t>, int> have;
    int dev = 0;
    SAQG_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    auto it = have.find({fn, dev, smem});
    if (it != have.end()) return it->second;
    int sms = 0, per_sm = 0;
    SAQG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SAQG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
    const int g = std::max(1, sms * std::max(1, per_sm));
    have[{fn, dev, smem}] = g;
    return g;
}

}  // namespace

int64_t tune_bucket(int64_t nq) {
    int64_t b = 1;
    while (b < nq) b <<= 1;
    return b;
}

void clamp_shape(const int *np, const int *k, int64_t nq, int np_max, int k_max, int *np_out, int *k_out,
                 cudaStream_t st) {
    if (nq <= 0 || (!np && !k)) return;
    k_clamp_shape<<<(unsigned)((nq + 255) / 256), 256, 0, st>>>(np, k, (int)nq, np_max, k_max, np_out, k_out);
    check_launch("k_clamp_shape");
    count_launch(1);
}

namespace {


// Centroid ranking of a batch: TF32 GEMM of inner products, the shortlist
// kernel, and the full exact path for the queries it hands back.
void probe_shortlist(const Index &I, SearchCtx &C, const float *q, int64_t nq, int64_t nprobe, const int *qnp,
                     float *dist, uint32_t *probe, uint8_t *full, int *fb_list, int *flags, Cand *work,
                     unsigned long long *cnt, void *qbf, cudaStream_t st,
                     const std::function<void()> &after_gemm = nullptr) {
    const DevIndexView &ix = I.view;
    {
        std::lock_guard<std::mutex> lk(I.init_mu);
        if (!I.cnorm2) {
            float *p = nullptr;
            SAQG_CUDA_TRY(cudaMalloc(&p, 8 * (size_t)I.K));
            k_cnorm2<<<(unsigned)((I.K * 32 + 255) / 256), 256, 0, st>>>(ix, reinterpret_cast<float2 *>(p));
            check_launch("k_cnorm2");
            SAQG_CUDA_TRY(cudaStreamSynchronize(st));  // other contexts read it on their own streams
            I.cnorm2 = p;
        }
    }
    {
        std::lock_guard<std::mutex> lk(I.init_mu);
        if (!I.cent_bf16) {
            void *p = nullptr;
            SAQG_CUDA_TRY(cudaMalloc(&p, 2 * (size_t)I.K * I.D));
            to_bf16(ix.centroids, I.K * I.D, p, st);
            SAQG_CUDA_TRY(cudaStreamSynchronize(st));  // other contexts read it on their own streams
            I.cent_bf16 = p;
        }
    }
    // dist (row-major nq x K) = Q C^T on the tensor cores (BF16 operands rounded
    // to nearest, FP32 accumulation); flags[3] is set if a GEMM wait timed out
    to_bf16(q, nq * I.D, qbf, st);
    probe_ip_gemm(qbf, nq, I.cent_bf16, I.K, I.D, dist, flags + 3, st);
    // Work that can run beside the shortlist and its select.  The caller's stream
    // has the device's least (default) priority, like that work's, so the shortlist
    // and the select then move to the context's greatest-priority stream: their CTAs
    // go first and the side work fills the gaps.
    cudaStream_t ps = st;
    if (after_gemm) {
        after_gemm();
        ps = C.aux_stream();
        SAQG_CUDA_TRY(cudaEventRecord(C.fork_event(), st));
        SAQG_CUDA_TRY(cudaStreamWaitEvent(ps, C.fork_event(), 0));
    }
    const double u = 1.0 / 16777216.0;
    ShortBound sb;
    // BF16 operands lie within 2^-9 of their values: |q.c error| <= (2^-8 + 2^-18) |q||c| + accumulation
    sb.e1 = (float)(2.0 * (1.0 / 256 + 1.0 / 262144 + (double)(I.D + 2) * u));
    sb.e2 = (float)((2.0 * (double)I.D + 32.0) * u);
    // upper-end keys kept in shared memory for the full radix select, which only
    // a query with nprobe > kShortThreads / 2 runs
    const bool keep = I.K <= kShortKeys && nprobe > kShortThreads / 2;
    const size_t smem = 12 * (size_t)kShortCap + 4 * (size_t)I.D + (keep ? 4 * (size_t)I.K : 0);
    SAQG_REQUIRE(smem <= 220 * 1024, "dimension too large for the probe shortlist's shared memory");
    ensure_smem((const void *)k_probe_shortlist, (size_t)smem);
    k_probe_shortlist<<<(unsigned)nq, kShortThreads, smem, ps>>>(ix, q, dist, reinterpret_cast<const float2 *>(I.cnorm2),
                                                                 sb, (int)nprobe, qnp, probe, full,
                                                                 fb_list, flags + 2, cnt, flags + 3, keep ? 1 : 0);
    check_launch("k_probe_shortlist");
    k_probe_dist_list<<<608, 256, 0, ps>>>(ix, q, dist, fb_list, flags + 2);
    check_launch("k_probe_dist_list");
    k_probe_select<<<(unsigned)nq, kSelThreads, 0, ps>>>(dist, (int)I.K, (int)nprobe, probe, work, flags, full, qnp);
    check_launch("k_probe_select");
    if (ps != st) {
        SAQG_CUDA_TRY(cudaEventRecord(C.join_event(), ps));
        SAQG_CUDA_TRY(cudaStreamWaitEvent(st, C.join_event(), 0));
    }
}

}  // namespace

void presize_ctx(const Index &I, SearchCtx &C, int64_t nq, int64_t topk, int64_t nprobe) {
    std::lock_guard<std::mutex> lock(C.mu);
    C.scratch_get(search_scratch_bytes(I, nq, topk, nprobe, false));
    const int64_t pos_cap = split_positions(I, nq * I.max_blocks_of_probes(nprobe));
    C.split_scratch_get(split_scratch_bytes(I, nq, topk, nprobe, pos_cap));
    C.aux_stream();
    C.fork_event();
    C.join_event();
    C.low_stream();
    C.qfork_event();
    C.qjoin_event();
}



size_t search_bytes_estimate(const Index &I, int64_t nq, int64_t topk, int64_t nprobe) {
    const int64_t max_pos = I.max_blocks_of_probes(nprobe);
    const int64_t pos_cap = split_positions(I, nq * max_pos);
    return search_scratch_bytes(I, nq, topk, nprobe, false) + split_scratch_bytes(I, nq, topk, nprobe, pos_cap);
}

void run_search(const Index &I, const float *q, int64_t nq, int64_t topk, int64_t nprobe, float m, uint32_t *ids,
                float *dists, int mem, cudaStream_t st, saqg_search_stats *stats, uint32_t *probes_out,
                const int *np_host, const int *k_host, SearchCtx *ctx, const SearchOpts *opts) {
    std::unique_ptr<CtxLease> lease;
    if (!ctx) {
        lease = std::make_unique<CtxLease>(I, st);  // locked; ordered after its previous call
        ctx = lease->c;
    }
    SearchCtx &C = *ctx;
    // per-query nprobe / k (host arrays): the scalars become their maxima
    int64_t sum_np = nq * nprobe;
    if (np_host || k_host) {
        int64_t npm = 0, km = 0;
        sum_np = 0;
        for (int64_t i = 0; i < nq; ++i) {
            const int a = np_host ? np_host[i] : (int)nprobe, b = k_host ? k_host[i] : (int)topk;
            SAQG_REQUIRE(a >= 1 && a <= I.K, "every nprobe must be in [1, number of clusters]");
            SAQG_REQUIRE(b >= 1 && b <= kMaxTopK, "every topk must be in [1, 4096]");
            npm = std::max<int64_t>(npm, a);
            km = std::max<int64_t>(km, b);
            sum_np += a;
        }
        if (np_host) nprobe = npm;
        if (k_host) topk = km;
    }
    SAQG_REQUIRE(nq >= 0 && topk >= 1 && topk <= kMaxTopK, "topk must be in [1, 4096]");
    SAQG_REQUIRE(nprobe >= 1 && nprobe <= I.K, "nprobe must be in [1, number of clusters]");
    if (nq == 0) return;
    const DevIndexView &ix = I.view;
    std::unique_lock<std::mutex> lock(C.mu, std::defer_lock);
    if (!lease) lock.lock();  // a caller's own context (graph, serving slot)
    const bool host = mem == SAQG_MEM_HOST;
    Bump bp{(char *)C.scratch_get(search_scratch_bytes(I, nq, topk, nprobe, host))};
    QueryShape qsh;
    qsh.np_max = (int)nprobe;
    qsh.k_max = (int)topk;
    if (np_host) {
        int *d = bp.take<int>(nq);
        SAQG_CUDA_TRY(cudaMemcpyAsync(d, np_host, 4 * (size_t)nq, cudaMemcpyHostToDevice, st));
        qsh.np = d;
    }
    if (k_host) {
        int *d = bp.take<int>(nq);
        SAQG_CUDA_TRY(cudaMemcpyAsync(d, k_host, 4 * (size_t)nq, cudaMemcpyHostToDevice, st));
        qsh.k = d;
    }
    if (!np_host && !k_host && opts && (opts->np_dev || opts->k_dev)) {  // device arrays: clamped copies
        int *dn = opts->np_dev ? bp.take<int>(nq) : nullptr;
        int *dk = opts->k_dev ? bp.take<int>(nq) : nullptr;
        clamp_shape(opts->np_dev, opts->k_dev, nq, (int)nprobe, (int)topk, dn, dk, st);
        qsh.np = dn;
        qsh.k = dk;
    }
    // launch shapes: the caller's, else the autotuner's choice for this shape, else built-in
    ScanTune tune;
    if (opts && opts->tune) {
        tune = *opts->tune;
    } else {
        std::lock_guard<std::mutex> lk(I.tune_mu);
        const auto it = I.scan_tunes.find(TuneKey{0, tune_bucket(nq), topk, nprobe});
        if (it != I.scan_tunes.end()) tune = it->second;
    }
    float *dq = bp.take<float>((size_t)nq * I.D);
    float *dist = bp.take<float>((size_t)nq * I.K);
    Cand *work = bp.take<Cand>((size_t)nq * I.K);
    uint32_t *probe = bp.take<uint32_t>((size_t)nq * nprobe);
    float *qrot = bp.take<float>((size_t)nq * ix.Dtot);
    float *prune = bp.take<float>((size_t)nq * ix.S);
    void *qbf = bp.take<uint16_t>((size_t)nq * I.D);
    uint8_t *full = bp.take<uint8_t>((size_t)nq);
    int *fb_list = bp.take<int>((size_t)nq);
    // heaviest queries first once the CTA scan runs in several waves
    int *order = nq >= kOrderMinQueries ? bp.take<int>((size_t)nq) : nullptr;
    uint32_t *oid = bp.take<uint32_t>((size_t)nq * topk);
    float *od = bp.take<float>((size_t)nq * topk);
    int *flags = bp.take<int>(16);
    unsigned long long *counters = bp.take<unsigned long long>(8);
    const int64_t pslots = prep_slots(I, nq, nprobe);
    uint16_t *prep_lut = pslots ? bp.take<uint16_t>((size_t)pslots * nprobe * 4 * ix.Dtot) : nullptr;
    SegScal *prep_scal = pslots ? bp.take<SegScal>((size_t)pslots * nprobe * ix.S) : nullptr;
    const bool scan_prep_fits = pslots > 0 && pslots == nq;
    uint16_t *scan_lut = scan_prep_fits ? bp.take<uint16_t>((size_t)nq * nprobe * 4 * ix.Dtot) : nullptr;
    SegScal *scan_scal = scan_prep_fits ? bp.take<SegScal>((size_t)nq * nprobe * ix.S) : nullptr;
    cudaEvent_t ev[7] = {};
    bool shortlist = false;  // centroid ranking by the GEMM shortlist
    if (stats)
        for (auto &e : ev) SAQG_CUDA_TRY(cudaEventCreate(&e));
    struct EvGuard {
        cudaEvent_t *e;
        ~EvGuard() {
            for (int i = 0; i < 7; ++i)
                if (e[i]) cudaEventDestroy(e[i]);
        }
    } evg{ev};
    const float *qin = q;
    if (host) {
        SAQG_CUDA_TRY(cudaMemcpyAsync(dq, q, 4 * (size_t)nq * I.D, cudaMemcpyHostToDevice, st));
        qin = dq;
    }
    SAQG_CUDA_TRY(cudaMemsetAsync(flags, 0, 64, st));
    if (stats) SAQG_CUDA_TRY(cudaMemsetAsync(counters, 0, 64, st));
    {
        const int wpb = 8;
        dim3 grid((unsigned)((I.K + wpb - 1) / wpb), (unsigned)nq);
        if (stats) SAQG_CUDA_TRY(cudaEventRecord(ev[0], st));
        // query preparation (rotation, prune bounds) depends on the queries alone:
        // it runs on the context's least-priority stream beside the centroid ranking
        // (beside the shortlist and its select when the GEMM ranks the centroids:
        // the GEMM wants whole SMs; those two then run at the greatest priority,
        // so their CTAs go first)
        auto launch_qprep = [&]() {
            cudaStream_t qs = C.low_stream();
            SAQG_CUDA_TRY(cudaEventRecord(C.qfork_event(), st));
            SAQG_CUDA_TRY(cudaStreamWaitEvent(qs, C.qfork_event(), 0));
            size_t qsm = 0;
            for (int s = 0; s < ix.S; ++s) qsm = std::max(qsm, (size_t)4 * ix.seg[s].dim);
            if (nq >= kQprepQT && kQprepQT * qsm <= 200 * 1024) {
                ensure_smem((const void *)k_qprep_tiled, (size_t)(kQprepQT * qsm));
                k_qprep_tiled<<<dim3((unsigned)ix.S, (unsigned)((nq + kQprepQT - 1) / kQprepQT),
                                     (unsigned)((qsm / 4 + kQprepSlice - 1) / kQprepSlice)),
                                kQprepSlice, kQprepQT * qsm, qs>>>(ix, qin, (int)nq, m, qrot, prune);
                check_launch("k_qprep_tiled");
            } else {
                int dmax = 0;
                for (int s = 0; s < ix.S; ++s) dmax = std::max(dmax, ix.seg[s].dim);
                const size_t sm_small = 4 * ((size_t)dmax + (size_t)(dmax / 16 + 1) * kQprepOut);
                k_qprep_small<<<dim3((unsigned)ix.S, (unsigned)nq, (unsigned)((dmax + kQprepOut - 1) / kQprepOut)),
                                256, sm_small, qs>>>(ix, qin, m, qrot, prune);
                check_launch("k_qprep_small");
            }
            SAQG_CUDA_TRY(cudaEventRecord(C.qjoin_event(), qs));
        };
        const char *pm = std::getenv("SAQG_PROBE");
        shortlist = nq >= kGemmMinQueries && nprobe <= kShortCap && !(pm && std::string(pm) == "exact");
        if (!shortlist) launch_qprep();
        if (shortlist) {
            probe_shortlist(I, C, qin, nq, nprobe, qsh.np, dist, probe, full, fb_list, flags, work,
                            stats ? counters : nullptr, qbf, st, launch_qprep);
        } else if (nq >= 8 && I.D % 32 == 0 && I.D <= 32 * kProbeRegs) {
            const size_t qsm = 4 * (size_t)kProbeQT * I.D;
            ensure_smem((const void *)k_probe_dist_tiled, (size_t)qsm);
            const unsigned gx = (unsigned)std::min<int64_t>((I.K + kProbeWarps - 1) / kProbeWarps, 304);
            k_probe_dist_tiled<<<dim3(gx, (unsigned)((nq + kProbeQT - 1) / kProbeQT)), kProbeWarps * 32, qsm, st>>>(
                ix, qin, (int)nq, dist);
            check_launch("k_probe_dist_tiled");
        } else {
            k_probe_dist<<<grid, wpb * 32, 0, st>>>(ix, qin, dist);
            check_launch("k_probe_dist");
        }
        if (!shortlist) {
            k_probe_select<<<(unsigned)nq, kSelThreads, 0, st>>>(dist, (int)I.K, (int)nprobe, probe, work, flags,
                                                                  nullptr, qsh.np);
            check_launch("k_probe_select");
        }
        if (stats) SAQG_CUDA_TRY(cudaEventRecord(ev[1], st));
        SAQG_CUDA_TRY(cudaStreamWaitEvent(st, C.qjoin_event(), 0));  // the rotated queries
        if (stats) SAQG_CUDA_TRY(cudaEventRecord(ev[2], st));
        const int xs = xstride_of(ix);
        const size_t smem = scan_smem_bytes(ix.Dtot, ix.S, (int)topk, xs);
        SAQG_REQUIRE(smem <= 200 * 1024, "dimension / topk too large for the scan kernel's shared memory");
        uint32_t *ids_out = host ? oid : ids;
        float *d_out = host ? od : dists;
        unsigned long long *cnt = stats ? counters : nullptr;
        const int mode0 = scan_mode(nq, topk, tune);
        const int mode = (qsh.np || qsh.k) && mode0 == 2 ? 0 : mode0;
        // The CTA scan's queries get batched LUTs too (by query; on the caller's stream,
        // after the split pass has forked, so it overlaps the split pass's start) when
        // the budget holds every query's: one batched kernel builds them for less than
        // the scan CTAs do (10M / 4,096 queries: 3.70 against 3.81 ms per batch).
        const std::function<Prepared(const uint8_t *)> scan_prep = [&](const uint8_t *skip) {  // skip: queries left out
            Prepared pp;
            if (!scan_lut || scan_ws(tune)) return pp;
            const size_t lsm = 4 * (size_t)kLutWarps * ix.Dtot;
            SAQG_REQUIRE(lsm <= 200 * 1024, "dimension too large for the batched LUT preparation");
            ensure_smem((const void *)k_lut, lsm);
            const int64_t items = nq * nprobe;
            k_lut<<<(unsigned)((items + kLutWarps - 1) / kLutWarps), kLutWarps * 32, lsm, st>>>(
                ix, probe, qsh, nullptr, nullptr, (int)nq, skip, qrot, prune, scan_lut, scan_scal);
            check_launch("k_lut");
            count_launch(1);
            pp.lut = scan_lut;
            pp.scal = scan_scal;
            pp.np_max = (int)nprobe;
            pp.slots = (int)nq;
            return pp;
        };

        if (mode == 2) {
            const size_t per_warp = align16(warp_smem_bytes(ix.Dtot, ix.S, (int)topk));
            const size_t wsm = per_warp * kWarpsPerCta;
            ensure_smem((const void *)k_scan_warp, (size_t)wsm);
            k_scan_warp<<<(unsigned)((nq + kWarpsPerCta - 1) / kWarpsPerCta), kWarpsPerCta * 32, wsm, st>>>(
                ix, probe, (int)nprobe, (int)nq, qrot, prune, (int)topk, ids_out, d_out, cnt, per_warp);
            check_launch("k_scan_warp");
            count_launch(4);
        } else if (mode == 0 && no_deferral(I, nprobe, tune)) {
            // no query of this call can probe more blocks than the deferral
            // threshold: the CTA scan answers every query, no split pass
            launch_cta_scan(scan_ws(tune), ix, probe, qsh, qrot, prune, ids_out, d_out, cnt, xs, nullptr, nq, order,
                            nullptr, scan_prep, st);
            count_launch(4);
        } else {
            // split-pass state: every query (mode 1), or the deferred giant-cluster queries (mode 0)
            const int64_t max_pos = I.max_blocks_of_probes(nprobe);
            const int64_t cap = nq;
            const int64_t want = nq * max_pos;
            const int64_t pos_cap = split_positions(I, want);
            Bump sb{(char *)C.split_scratch_get(split_scratch_bytes(I, cap, topk, nprobe, pos_cap))};
            SplitState ss;
            ss.nlist = sb.take<int>(16);
            ss.pos_used = reinterpret_cast<unsigned long long *>(ss.nlist + 2);
            ss.work_next = ss.nlist + 4;
            ss.qlist = sb.take<int>(cap);
            ss.cap = (int)cap;
            ss.pool_id = sb.take<uint32_t>((size_t)cap * topk);
            ss.pool_d = sb.take<float>((size_t)cap * topk);
            ss.pool_size = sb.take<int>(cap);
            ss.tau = sb.take<float>(cap);
            ss.tile_off = sb.take<int>((size_t)cap * (nprobe + 1));
            ss.blk_base = sb.take<int>((size_t)cap * nprobe);
            ss.split_p = sb.take<int>(cap);
            ss.split_b = sb.take<int>(cap);
            ss.q_tile_off = sb.take<int>(cap + 1);
            ss.npos = sb.take<int>(cap);
            ss.pos_off = sb.take<int64_t>(cap);
            ss.pos_cap = pos_cap;
            ss.summ = sb.take<float4>((size_t)pos_cap);
            ss.rec_words = rec_words_of(ix.S);
            ss.rec = sb.take<float>((size_t)pos_cap * ss.rec_words);
            ss.qsh = qsh;
            // heavy queries beside a batch: a longer prefix for a tighter bound; a
            // few queries alone: the speculative part has the GPU, so only the pool must fill
            ss.first_blocks = tune.first_blocks > 0 ? tune.first_blocks : (mode == 0 ? kFirstBlocks : 1);
            ss.t_lo = 0;
            ss.t_hi = INT_MAX;
            ss.final_level = 1;
            if (const char *e = std::getenv("SAQG_FIRST_BLOCKS")) ss.first_blocks = std::max(1, std::atoi(e));
            uint8_t *deferred = sb.take<uint8_t>(nq);
            int *qblocks = sb.take<int>(nq);
            SAQG_CUDA_TRY(cudaMemsetAsync(ss.summ, 0xff, 16 * (size_t)pos_cap, st));  // NaN: no record
            SAQG_CUDA_TRY(cudaMemsetAsync(ss.nlist, 0, 32, st));
            int defer = -1;  // mode 1: every query
            if (mode == 0) defer = defer_threshold(tune);
            const int dthreads = (int)std::min<int64_t>(kDeferThreads, (nq + 31) / 32 * 32);
            const bool par = nq >= kQblocksMinQueries;
            if (par) {
                k_qblocks<<<(unsigned)((nq + 255) / 256), 256, 0, st>>>(ix, probe, qsh, (int)nq, qblocks);
                check_launch("k_qblocks");
            }
            k_defer<<<1, dthreads, 0, st>>>(ix, probe, (int)nq, defer, ss, qblocks, par ? 1 : 0, deferred);
            check_launch("k_defer");
            cudaStream_t sp = st;  // stream of the split pass
            // the CTA scan serves what the split list does not hold: always in mode 0,
            // in mode 1 only when the record space cannot hold every query
            if (mode == 0 || pos_cap < want) {
                if (mode == 0) {  // the split pass runs beside the CTA scan on the index's auxiliary stream
                    sp = C.aux_stream();
                    SAQG_CUDA_TRY(cudaEventRecord(C.fork_event(), st));
                    SAQG_CUDA_TRY(cudaStreamWaitEvent(sp, C.fork_event(), 0));
                }
                launch_cta_scan(scan_ws(tune), ix, probe, qsh, qrot, prune, ids_out, d_out, cnt, xs, deferred, nq,
                                order, qblocks, scan_prep, st);
            }
            const size_t smem1 = scan_smem_bytes(ix.Dtot, ix.S, 1, xs);
            const size_t smem_r = smem + 2 * 4 * (size_t)kReplayRecs * ss.rec_words;
            SAQG_REQUIRE(smem_r <= 220 * 1024, "dimension / topk too large for the replay kernel's shared memory");
            ensure_smem((const void *)k_scan_first, (size_t)smem);
            ensure_smem((const void *)k_scan_spec, (size_t)smem1);
            ensure_smem((const void *)k_scan_replay, (size_t)smem_r);
            Prepared prep;  // the listed queries' LUTs, one batched kernel ahead of the split pass
            if (prep_lut) {
                const size_t lsm = 4 * (size_t)kLutWarps * ix.Dtot;
                SAQG_REQUIRE(lsm <= 200 * 1024, "dimension too large for the batched LUT preparation");
                ensure_smem((const void *)k_lut, lsm);
                const int64_t items = pslots * nprobe;
                k_lut<<<(unsigned)((items + kLutWarps - 1) / kLutWarps), kLutWarps * 32, lsm, sp>>>(
                    ix, probe, qsh, ss.qlist, ss.nlist, (int)pslots, nullptr, qrot, prune, prep_lut, prep_scal);
                check_launch("k_lut");
                count_launch(1);
                prep.lut = prep_lut;
                prep.scal = prep_scal;
                prep.np_max = (int)nprobe;
                prep.slots = (int)pslots;
            }
            // the list holds at most cap slots; the per-slot kernels loop over them
            const unsigned slot_grid = (unsigned)std::min<int64_t>(cap, 4 * (int64_t)sm_count());
            k_scan_first<<<slot_grid, kScanThreads, smem, sp>>>(ix, probe, qrot, prune, ss, flags + 1, cnt, xs,
                                                                     prep);
            check_launch("k_scan_first");
            if (stats) SAQG_CUDA_TRY(cudaEventRecord(ev[5], sp));
            const unsigned grid = (unsigned)full_grid((const void *)k_scan_spec, kScanThreads, smem1);
            // levels of speculation (tiles after the split point): each level's
            // replay leaves the exact pool, whose distk bounds the next level
            const int *levels = kSpecLevelSets[tune.spec_levels >= 0 && tune.spec_levels < kNumSpecLevelSets
                                                   ? tune.spec_levels : 0];
            int nlev = 1;
            if (mode == 0)
                while (nlev < kMaxSpecLevels && levels[nlev] >= 0) ++nlev;
            for (int L = 0; L < nlev; ++L) {
                SplitState sl = ss;
                sl.t_lo = mode == 0 ? levels[L] : 0;
                sl.t_hi = L + 1 < nlev ? levels[L + 1] : INT_MAX;
                sl.final_level = L + 1 == nlev;
                k_tile_prefix<<<1, kPrefixThreads, 0, sp>>>(sl);
                check_launch("k_tile_prefix");
                k_scan_spec<<<grid, kScanThreads, smem1, sp>>>(ix, probe, (int)nprobe, qrot, prune, sl, cnt, xs, prep);
                check_launch("k_scan_spec");
                if (stats && sl.final_level) SAQG_CUDA_TRY(cudaEventRecord(ev[6], sp));
                k_scan_replay<<<slot_grid, kScanThreads, smem_r, sp>>>(ix, sl, ids_out, d_out, cnt, xs);
                check_launch("k_scan_replay");
            }
            if (stats) SAQG_CUDA_TRY(cudaEventRecord(ev[4], sp));
            if (sp != st) {  // join
                SAQG_CUDA_TRY(cudaEventRecord(C.join_event(), sp));
                SAQG_CUDA_TRY(cudaStreamWaitEvent(st, C.join_event(), 0));
            }
            count_launch(mode == 0 ? 8 : 8);
        }
        if (stats) SAQG_CUDA_TRY(cudaEventRecord(ev[3], st));
    }
    if (probes_out)
        SAQG_CUDA_TRY(cudaMemcpyAsync(probes_out, probe, 4 * (size_t)nq * nprobe,
                                      host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st));
    if (host) {
        SAQG_CUDA_TRY(cudaMemcpyAsync(ids, oid, 4 * (size_t)nq * topk, cudaMemcpyDeviceToHost, st));
        if (dists) SAQG_CUDA_TRY(cudaMemcpyAsync(dists, od, 4 * (size_t)nq * topk, cudaMemcpyDeviceToHost, st));
        int hflags[2] = {0, 0};
        SAQG_CUDA_TRY(cudaMemcpyAsync(hflags, flags, 8, cudaMemcpyDeviceToHost, st));
        SAQG_CUDA_TRY(cudaStreamSynchronize(st));
        if (hflags[1]) throw Error{SAQG_ERR_INTERNAL, "scan replay met a lane without a precomputed distance"};
    }
    if (stats) {
        unsigned long long hc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        SAQG_CUDA_TRY(cudaMemcpyAsync(hc, counters, 64, cudaMemcpyDeviceToHost, st));
        SAQG_CUDA_TRY(cudaStreamSynchronize(st));
        float t01 = 0, t12 = 0, t23 = 0, t03 = 0;
        SAQG_CUDA_TRY(cudaEventElapsedTime(&t01, ev[0], ev[1]));
        SAQG_CUDA_TRY(cudaEventElapsedTime(&t12, ev[1], ev[2]));
        SAQG_CUDA_TRY(cudaEventElapsedTime(&t23, ev[2], ev[3]));
        SAQG_CUDA_TRY(cudaEventElapsedTime(&t03, ev[0], ev[3]));
        stats->ms_probe = t01;
        stats->ms_qprep = t12;
        stats->ms_scan = t23;
        stats->ms_total = t03;
        // split pass phases (0 when the call had no split pass)
        auto span = [&](int a, int b) {
            float t = 0.0f;
            if (cudaEventQuery(ev[a]) != cudaSuccess || cudaEventQuery(ev[b]) != cudaSuccess) return 0.0f;
            return cudaEventElapsedTime(&t, ev[a], ev[b]) == cudaSuccess ? t : 0.0f;
        };
        stats->ms_split = span(2, 4);
        stats->ms_split_first = span(2, 5);
        stats->ms_split_spec = span(5, 6);
        stats->ms_split_replay = span(6, 4);
        cudaGetLastError();
        stats->probes = sum_np;
        stats->blocks = (int64_t)hc[0];
        stats->vectors = (int64_t)hc[1];
        stats->reranked = (int64_t)hc[2];
        stats->speculative = (int64_t)hc[3];
        stats->probe_exact = shortlist ? (int64_t)hc[4] : nq * I.K;
        stats->probe_full = shortlist ? (int64_t)(hc[5] + hc[6]) : nq;
        stats->probe_full_ties = (int64_t)hc[6];
        // Algorithmic bytes: per scanned block 32 lanes of 1-bit codes of
        // every coded segment and |o| of every segment; per probe the rotated centroid;
        // per re-ranked vector its ex-codes, ex factors and id.
        int64_t per_lane = 0, per_rr = 4;
        for (int s = 0; s < ix.S; ++s) {
            per_lane += 4 + (ix.seg[s].bits ? ix.seg[s].dim / 8 : 0);
            per_rr += ix.seg[s].pv + 8;
        }
        stats->fast_bytes = stats->blocks * 32 * per_lane + stats->probes * 4 * (int64_t)ix.Dtot;
        stats->rerank_bytes = stats->reranked * per_rr;
    }
}

int64_t run_estimate(const Index &I, const float *q_host, int64_t nprobe, float m, uint32_t *ids, float *acc,
                     float *fast, float *vars, int64_t cap) {
    SAQG_REQUIRE(nprobe >= 1 && nprobe <= I.K, "nprobe must be in [1, number of clusters]");
    const DevIndexView &ix = I.view;
    cudaStream_t st = 0;
    CtxLease lease(I, st);
    Bump bp{(char *)lease.c->scratch_get(search_scratch_bytes(I, 1, 1, nprobe, true))};
    float *dq = bp.take<float>(I.D);
    float *dist = bp.take<float>(I.K);
    Cand *work = bp.take<Cand>(I.K);
    uint32_t *probe = bp.take<uint32_t>(nprobe);
    float *qrot = bp.take<float>(ix.Dtot);
    float *prune = bp.take<float>(ix.S);
    bp.take<uint32_t>(2);
    bp.take<float>(2);
    int *flags = bp.take<int>(16);
    SAQG_CUDA_TRY(cudaMemcpy(dq, q_host, 4 * I.D, cudaMemcpyHostToDevice));
    SAQG_CUDA_TRY(cudaMemset(flags, 0, 64));
    const int wpb = 8;
    k_probe_dist<<<dim3((unsigned)((I.K + wpb - 1) / wpb), 1), wpb * 32, 0, st>>>(ix, dq, dist);
    check_launch("k_probe_dist");
    k_probe_select<<<1, kSelThreads, 0, st>>>(dist, (int)I.K, (int)nprobe, probe, work, flags);
    check_launch("k_probe_select");
    size_t qsm = 0;
    for (int s = 0; s < ix.S; ++s) qsm = std::max(qsm, (size_t)4 * ix.seg[s].dim);
    k_qprep<<<dim3((unsigned)ix.S, 1), 256, qsm, st>>>(ix, dq, m, qrot, prune);
    check_launch("k_qprep");
    std::vector<uint32_t> hprobe(nprobe);
    SAQG_CUDA_TRY(cudaMemcpy(hprobe.data(), probe, 4 * nprobe, cudaMemcpyDeviceToHost));
    std::vector<int64_t> off(nprobe + 1, 0);
    for (int64_t p = 0; p < nprobe; ++p) off[p + 1] = off[p] + I.sizes[hprobe[p]];
    const int64_t total = off[nprobe];
    if (total > 0) {
        int64_t *doff;
        uint32_t *oids;
        float *oacc, *ofast, *ovars;
        SAQG_CUDA_TRY(cudaMalloc(&doff, 8 * (nprobe + 1)));
        SAQG_CUDA_TRY(cudaMalloc(&oids, 4 * total));
        SAQG_CUDA_TRY(cudaMalloc(&oacc, 4 * total));
        SAQG_CUDA_TRY(cudaMalloc(&ofast, 4 * total));
        SAQG_CUDA_TRY(cudaMalloc(&ovars, 4 * total));
        SAQG_CUDA_TRY(cudaMemcpy(doff, off.data(), 8 * (nprobe + 1), cudaMemcpyHostToDevice));
        const int xs = xstride_of(ix);
        const size_t smem = scan_smem_bytes(ix.Dtot, ix.S, 1, xs);
        ensure_smem((const void *)k_estimate, (size_t)smem);
        k_estimate<<<(unsigned)nprobe, kScanThreads, smem, st>>>(ix, probe, doff, qrot, prune, oids, oacc, ofast, ovars,
                                                                 xs);
        check_launch("k_estimate");
        count_launch(4);
        const int64_t nw = std::min(total, cap);
        SAQG_CUDA_TRY(cudaMemcpy(ids, oids, 4 * nw, cudaMemcpyDeviceToHost));
        SAQG_CUDA_TRY(cudaMemcpy(acc, oacc, 4 * nw, cudaMemcpyDeviceToHost));
        SAQG_CUDA_TRY(cudaMemcpy(fast, ofast, 4 * nw, cudaMemcpyDeviceToHost));
        SAQG_CUDA_TRY(cudaMemcpy(vars, ovars, 4 * nw, cudaMemcpyDeviceToHost));
        cudaFree(doff);
        cudaFree(oids);
        cudaFree(oacc);
        cudaFree(ofast);
        cudaFree(ovars);
    }
    return total;
}

// ------------------------------------------------- search with static scratch
// The scratch of saqg_search_static: one file-scope device array (one instance
// per device, placed by the driver when it loads this file's kernels), shared by
// every call on that device.  Nothing in it needs to start at zero except the
// 64-byte flag words, which each call clears on its stream before its kernels.
// Because it belongs to this file's module, every process that runs any search
// kernel of the library on a device holds these 16 MiB there until it exits,
// whether or not it calls saqg_search_static.
static __device__ __align__(256) unsigned char g_static_scratch[SAQG_STATIC_SCRATCH_BYTES];

namespace {

constexpr int kMaxStaticDevices = 64;
std::mutex g_static_mu;
void *g_static_ptr[kMaxStaticDevices] = {};

// Device address of the array on `dev` (current), looked up on the first call
// on that device.
void *static_scratch(int dev) {
    SAQG_REQUIRE(dev >= 0 && dev < kMaxStaticDevices, "device ordinal out of range for the static scratch");
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p)
            throw Error{SAQG_ERR_CUDA, std::string("cudaGetSymbolAddress(static scratch) failed: ") +
                                           cudaGetErrorString(e)};
        g_static_ptr[dev] = p;
    }
    return g_static_ptr[dev];
}

}  // namespace

size_t static_search_scratch_bytes(const Index &I, int64_t nq, int64_t nprobe) {
    size_t b = 0;
    auto add = [&](size_t x) { b += align16(x); };
    add(4 * (size_t)nq * I.K);          // centroid distances
    add(8 * (size_t)nq * I.K);          // exact-select work (fallback)
    add(4 * (size_t)nq * nprobe);       // probe ids
    add(4 * (size_t)nq * I.view.Dtot);  // rotated queries
    add(4 * (size_t)nq * I.view.S);     // prune bounds
    add(64);                            // flags
    return b;
}

void run_search_static(const Index &I, const float *q, int64_t nq, int64_t topk, int64_t nprobe, float m,
                       uint32_t *ids, float *dists, cudaStream_t st) {
    SAQG_REQUIRE(nq >= 0 && topk >= 1 && topk <= kMaxTopK, "topk must be in [1, 4096]");
    SAQG_REQUIRE(nprobe >= 1 && nprobe <= I.K, "nprobe must be in [1, number of clusters]");
    if (nq == 0) return;
    const size_t need = static_search_scratch_bytes(I, nq, nprobe);
    SAQG_REQUIRE(need <= (size_t)SAQG_STATIC_SCRATCH_BYTES,
                 "saqg_search_static: " + std::to_string(nq) + " queries with " + std::to_string(I.K) +
                     " clusters and nprobe " + std::to_string(nprobe) + " need " + std::to_string(need) +
                     " bytes of scratch, above the static maximum of " +
                     std::to_string((size_t)SAQG_STATIC_SCRATCH_BYTES) + " bytes; split the batch");
    // The kernels would fault on a host pointer or one on another device; a
    // wrong pointer is reported instead (this call takes device memory only).
    auto require_device_ptr = [&](const void *p, const char *what) {
        cudaPointerAttributes a{};
        const cudaError_t e = cudaPointerGetAttributes(&a, p);
        if (e != cudaSuccess) {
            cudaGetLastError();
            throw Error{SAQG_ERR_INVALID, std::string("saqg_search_static: ") + what +
                                              " is not a pointer the CUDA runtime knows: " + cudaGetErrorString(e)};
        }
        if (a.type == cudaMemoryTypeManaged) return;
        if (a.type != cudaMemoryTypeDevice || a.device != I.device)
            throw Error{SAQG_ERR_INVALID, std::string("saqg_search_static: ") + what +
                                              " must be device memory on the index's device (" +
                                              std::to_string(I.device) + ")"};
    };
    require_device_ptr(q, "queries");
    require_device_ptr(ids, "ids");
    if (dists) require_device_ptr(dists, "dists");
    const DevIndexView &ix = I.view;
    const size_t smem = scan_smem_bytes(ix.Dtot, ix.S, (int)topk, xstride_of(ix));
    SAQG_REQUIRE(smem <= 200 * 1024, "dimension / topk too large for the scan kernel's shared memory");
    int prev = 0;
    SAQG_CUDA_TRY(cudaGetDevice(&prev));
    struct DevGuard {
        int prev, cur;
        ~DevGuard() {
            if (prev != cur) cudaSetDevice(prev);
        }
    } dg{prev, I.device};
    if (prev != I.device) SAQG_CUDA_TRY(cudaSetDevice(I.device));
    Bump bp{(char *)static_scratch(I.device)};
    float *dist = bp.take<float>((size_t)nq * I.K);
    Cand *work = bp.take<Cand>((size_t)nq * I.K);
    uint32_t *probe = bp.take<uint32_t>((size_t)nq * nprobe);
    float *qrot = bp.take<float>((size_t)nq * ix.Dtot);
    float *prune = bp.take<float>((size_t)nq * ix.S);
    int *flags = bp.take<int>(16);
    SAQG_CUDA_TRY(cudaMemsetAsync(flags, 0, 64, st));
    if (nq >= 8 && I.D % 32 == 0 && I.D <= 32 * kProbeRegs) {
        const size_t qsm = 4 * (size_t)kProbeQT * I.D;
        ensure_smem((const void *)k_probe_dist_tiled, (size_t)qsm);
        const unsigned gx = (unsigned)std::min<int64_t>((I.K + kProbeWarps - 1) / kProbeWarps, 304);
        k_probe_dist_tiled<<<dim3(gx, (unsigned)((nq + kProbeQT - 1) / kProbeQT)), kProbeWarps * 32, qsm, st>>>(
            ix, q, (int)nq, dist);
        check_launch("k_probe_dist_tiled");
    } else {
        const int wpb = 8;
        k_probe_dist<<<dim3((unsigned)((I.K + wpb - 1) / wpb), (unsigned)nq), wpb * 32, 0, st>>>(ix, q, dist);
        check_launch("k_probe_dist");
    }
    k_probe_select<<<(unsigned)nq, kSelThreads, 0, st>>>(dist, (int)I.K, (int)nprobe, probe, work, flags);
    check_launch("k_probe_select");
    size_t qsm = 0;
    for (int s = 0; s < ix.S; ++s) qsm = std::max(qsm, (size_t)4 * ix.seg[s].dim);
    k_qprep<<<dim3((unsigned)ix.S, (unsigned)nq), 256, qsm, st>>>(ix, q, m, qrot, prune);
    check_launch("k_qprep");
    const size_t smem_k = scan_smem_bytes(ix.Dtot, ix.S, (int)topk, xstride_of(ix));
    SAQG_REQUIRE(smem_k <= 200 * 1024, "dimension / topk too large for the scan kernel's shared memory");
    ensure_smem((const void *)k_scan, (size_t)smem_k);
    QueryShape qsh;
    qsh.np_max = (int)nprobe;
    qsh.k_max = (int)topk;
    k_scan<<<(unsigned)nq, kScanThreads, smem_k, st>>>(ix, probe, qsh, qrot, prune, ids, dists, nullptr,
                                                      xstride_of(ix), nullptr, nullptr, Prepared{});
    check_launch("k_scan");
    count_launch(4);
}

// ------------------------------------------ tensor-core form: probes and re-rank
namespace {

// Distance the search inserts for a vector that passes every pruning stage
// (block_estimates + the accurate pass + replay_block): one segment, the
// accurate distance; several, the running sum of variance bounds, each coded
// segment's bound replaced by its fast estimate, then every segment's
// estimate replaced by its accurate distance, in segment order.
__device__ float searched_dist(const DevIndexView &ix, const ScanSmem &sm, int64_t gb, int64_t gv, int ln, int lane) {
    const int S = ix.S;
    float v[kMaxSeg], f[kMaxSeg], ipx[kMaxSeg];
    for (int s = 0; s < S; ++s) {
        const SegDev &g = ix.seg[s];
        const float on = g.onorm[gb * 32 + lane];
        v[s] = vars_est(sm.scal[s], on);
        float ip = 0.0f;
        f[s] = g.bits ? fast_est(g, sm.lut + 4 * g.qoff, sm.scal[s], gb, lane, on, ip) : v[s];
        ipx[s] = __shfl_sync(kFull, ip, ln);
        v[s] = __shfl_sync(kFull, v[s], ln);
        f[s] = __shfl_sync(kFull, f[s], ln);
    }
    // ex-code inner products by the 16 lanes of CodeHelper::compute_ip (each
    // half-warp computes them; lane 0 holds the result)
    float ex[kMaxSeg];
    const unsigned half = lane < 16 ? 0x0000ffffu : 0xffff0000u;
    for (int s = 0; s < S; ++s) {
        const SegDev &g = ix.seg[s];
        ex[s] = g.bits > 1 ? excode_ip_half(sm.qres + g.qoff, g.lcode + (size_t)gv * g.lstride, g.dim, g.bits - 1,
                                            lane & 15, half)
                           : 0.0f;
    }
    float d = 0.0f;
    if (lane == 0) {
        float acc[kMaxSeg];
        for (int s = 0; s < S; ++s) {
            const SegDev &g = ix.seg[s];
            acc[s] = accurate_dist(g.onorm[gb * 32 + ln], ipx[s], ex[s], g.exfac[gv].x, g.bits, sm.scal[s].sum_q,
                                   sm.scal[s].q_l2sqr);
        }
        if (S == 1) {
            d = acc[0];
        } else {
            float cur = 0.0f;
            for (int s = 0; s < S; ++s) cur = __fadd_rn(cur, v[s]);
            for (int s = 0; s < S; ++s)
                if (ix.seg[s].bits) cur = __fadd_rn(__fsub_rn(cur, v[s]), f[s]);
            d = cur;
            for (int s = 0; s < S; ++s) d = __fadd_rn(d, __fsub_rn(acc[s], ix.seg[s].bits ? f[s] : v[s]));
        }
    }
    return __shfl_sync(kFull, d, 0);
}

// Groups of a query's shortlist (positions ascending, so grouped by probe):
// the first entry and the probe index of each probed cluster holding
// shortlisted vectors.  One thread per query.
__global__ void k_tc_groups(const int *__restrict__ sl_pos, const int *__restrict__ sl_cnt,
                            const int *__restrict__ lp, int nq, int nprobe, int L, int *__restrict__ grp,
                            int *__restrict__ gj, int *__restrict__ ng) {
    const int qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    const int n = sl_cnt[qi];
    const int *pos = sl_pos + (size_t)qi * L;
    const int *lq = lp + (size_t)qi * (nprobe + 1);
    int cnt = 0, j = 0;
    for (int e = 0; e < n; ++e) {
        if (e > 0 && pos[e] < lq[j + 1]) continue;  // same probe as the previous entry
        while (lq[j + 1] <= pos[e]) ++j;           // probes are visited in order
        grp[(size_t)qi * L + cnt] = e;
        gj[(size_t)qi * L + cnt] = j;
        ++cnt;
    }
    ng[qi] = cnt;
}

// Re-rank of the tensor-core shortlist: CTA (g, query) takes the query's g-th
// group, i.e. one probed cluster: Lut::prepare for it, then the distance the
// search computes (searched_dist) of each of its shortlisted vectors.
__global__ void __launch_bounds__(kScanThreads) k_tc_rerank(DevIndexView ix, const uint32_t *__restrict__ probe,
                                                            int nprobe, const float *__restrict__ qrot,
                                                            const float *__restrict__ prune,
                                                            const int *__restrict__ lp, const int *__restrict__ sl_pos,
                                                            const int *__restrict__ sl_cnt, const int *__restrict__ grp,
                                                            const int *__restrict__ gj, const int *__restrict__ ng,
                                                            int L, float *__restrict__ sl_dist) {
    extern __shared__ __align__(16) char smem_raw[];
    const int qi = blockIdx.y, g = blockIdx.x;
    const int ngq = ng[qi];
    if (g >= ngq) return;
    ScanSmem sm = scan_smem_layout(smem_raw, ix.Dtot, ix.S, 1, 0);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g0 = grp[(size_t)qi * L + g], g1 = g + 1 < ngq ? grp[(size_t)qi * L + g + 1] : sl_cnt[qi];
    const int j = gj[(size_t)qi * L + g];
    const int base = lp[(size_t)qi * (nprobe + 1) + j];
    const int c = (int)probe[(size_t)qi * nprobe + j];
    prepare_cluster(ix, qrot + (size_t)qi * ix.Dtot, prune + (size_t)qi * ix.S, c, sm);
    const int64_t b0 = ix.blk_off[c], v0 = ix.vec_off[c];
    const int *pos = sl_pos + (size_t)qi * L;
    for (int e = g0 + w; e < g1; e += kScanWarps) {
        const int r = pos[e] - base;
        const float d = searched_dist(ix, sm, b0 + r / 32, v0 + r, r & 31, lane);
        if (lane == 0) sl_dist[(size_t)qi * L + e] = d;
    }
}

// Top-k of the re-ranked shortlist, one CTA per query: ordered by distance,
// equal distances the later-scanned first, which is where ResultPool::insert
// puts an equal distance (pool.hpp:17-30).
__global__ void __launch_bounds__(kScanThreads) k_tc_topk(DevIndexView ix, const uint32_t *__restrict__ probe,
                                                          int nprobe, const int *__restrict__ lp,
                                                          const int *__restrict__ sl_pos,
                                                          const float *__restrict__ sl_apx,
                                                          const int *__restrict__ sl_cnt,
                                                          const float *__restrict__ sl_dist, int L, int L2, int topk,
                                                          const int *__restrict__ qk, uint32_t *__restrict__ ids,
                                                          float *__restrict__ dists, float *__restrict__ apx_out) {
    extern __shared__ __align__(16) char smem_raw[];
    unsigned long long *key = reinterpret_cast<unsigned long long *>(smem_raw);
    const int qi = blockIdx.x, tid = threadIdx.x;
    const int n = sl_cnt[qi];
    const int *pos = sl_pos + (size_t)qi * L;
    const float *dist = sl_dist + (size_t)qi * L;
    const int *lq = lp + (size_t)qi * (nprobe + 1);
    for (int e = tid; e < L2; e += blockDim.x)
        key[e] = e < n ? ((unsigned long long)fkey(dist[e]) << 32) | (unsigned)(0x7fffffff - pos[e]) : ~0ull;
    __syncthreads();
    for (int k = 2; k <= L2; k <<= 1)
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            for (int e = tid; e < L2; e += blockDim.x) {
                const int o = e ^ jj;
                if (o > e) {
                    const unsigned long long a = key[e], b = key[o];
                    if ((a > b) == ((e & k) == 0)) {
                        key[e] = b;
                        key[o] = a;
                    }
                }
            }
            __syncthreads();
        }
    const int kq = qk ? qk[qi] : topk;  // this query's k; rows are topk long, padded with (0, FLT_MAX)
    for (int t = tid; t < topk; t += blockDim.x) {
        uint32_t id = 0;
        float d = FLT_MAX, a = FLT_MAX;
        if (t < n && t < kq) {
            const int p = 0x7fffffff - (int)(unsigned)(key[t] & 0xffffffffull);
            int lo = 0, hi = n - 1;  // the shortlist entry of position p
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (pos[mid] < p) lo = mid + 1;
                else hi = mid;
            }
            int jlo = 0, jhi = nprobe - 1;  // its probe: the last j with lq[j] <= p
            while (jlo < jhi) {
                const int mid = (jlo + jhi + 1) >> 1;
                if (lq[mid] <= p) jlo = mid;
                else jhi = mid - 1;
            }
            const int c = (int)probe[(size_t)qi * nprobe + jlo];
            id = ix.ids[ix.vec_off[c] + (p - lq[jlo])];
            d = dist[lo];
            a = sl_apx[(size_t)qi * L + lo];
        }
        ids[(size_t)qi * topk + t] = id;
        if (dists) dists[(size_t)qi * topk + t] = d;
        if (apx_out) apx_out[(size_t)qi * topk + t] = a;
    }
}

}  // namespace

void tc_rank_rotate(const Index &I, SearchCtx &C, const float *q, int64_t nq, int64_t nprobe, const int *qnp, float m,
                    float *dist, void *work, uint32_t *probe, float *qrot, float *prune, uint8_t *full, int *fb_list,
                    int *flags, void *qbf, cudaStream_t st) {
    const DevIndexView &ix = I.view;
    SAQG_CUDA_TRY(cudaMemsetAsync(flags, 0, 64, st));
    Cand *wk = static_cast<Cand *>(work);
    const char *pm = std::getenv("SAQG_PROBE");
    const bool shortlist = nq >= kGemmMinQueries && nprobe <= kShortCap && !(pm && std::string(pm) == "exact");
    if (shortlist) {
        probe_shortlist(I, C, q, nq, nprobe, qnp, dist, probe, full, fb_list, flags, wk, nullptr, qbf, st);
    } else {
        k_probe_dist<<<dim3((unsigned)((I.K + 7) / 8), (unsigned)nq), 256, 0, st>>>(ix, q, dist);
        check_launch("k_probe_dist");
        k_probe_select<<<(unsigned)nq, kSelThreads, 0, st>>>(dist, (int)I.K, (int)nprobe, probe, wk, flags, nullptr,
                                                              qnp);
        check_launch("k_probe_select");
    }
    size_t qsm = 0;
    for (int s = 0; s < ix.S; ++s) qsm = std::max(qsm, (size_t)4 * ix.seg[s].dim);
    if (nq >= kQprepQT && kQprepQT * qsm <= 200 * 1024) {
        ensure_smem((const void *)k_qprep_tiled, (size_t)(kQprepQT * qsm));
        k_qprep_tiled<<<dim3((unsigned)ix.S, (unsigned)((nq + kQprepQT - 1) / kQprepQT),
                             (unsigned)((qsm / 4 + kQprepSlice - 1) / kQprepSlice)),
                        kQprepSlice, kQprepQT * qsm, st>>>(ix, q, (int)nq, m, qrot, prune);
        check_launch("k_qprep_tiled");
    } else {
        k_qprep<<<dim3((unsigned)ix.S, (unsigned)nq), 256, qsm, st>>>(ix, q, m, qrot, prune);
        check_launch("k_qprep");
    }
    count_launch(4);
}

size_t tc_probe_work_bytes(const Index &I, int64_t nq) { return sizeof(Cand) * (size_t)nq * I.K; }

void tc_rerank(const Index &I, const uint32_t *probe, int64_t nq, int64_t nprobe, const float *qrot,
               const float *prune, const int *lp, const int *sl_pos, const float *sl_apx, const int *sl_cnt, int L,
               int64_t topk, const int *qk, int *grp, int *gj, int *ng, float *sl_dist, uint32_t *ids, float *dists,
               float *apx, cudaStream_t st) {
    const DevIndexView &ix = I.view;
    int L2 = 1;
    while (L2 < L) L2 <<= 1;
    k_tc_groups<<<(unsigned)((nq + 127) / 128), 128, 0, st>>>(sl_pos, sl_cnt, lp, (int)nq, (int)nprobe, L, grp, gj,
                                                               ng);
    check_launch("k_tc_groups");
    const size_t smem = scan_smem_bytes(ix.Dtot, ix.S, 1, 0);
    SAQG_REQUIRE(smem <= 200 * 1024, "dimension too large for the re-rank kernel's shared memory");
    ensure_smem((const void *)k_tc_rerank, (size_t)smem);
    k_tc_rerank<<<dim3((unsigned)L, (unsigned)nq), kScanThreads, smem, st>>>(ix, probe, (int)nprobe, qrot, prune, lp,
                                                                             sl_pos, sl_cnt, grp, gj, ng, L, sl_dist);
    check_launch("k_tc_rerank");
    k_tc_topk<<<(unsigned)nq, kScanThreads, 8 * (size_t)L2, st>>>(ix, probe, (int)nprobe, lp, sl_pos, sl_apx, sl_cnt,
                                                                  sl_dist, L, L2, (int)topk, qk, ids, dists, apx);
    check_launch("k_tc_topk");
    count_launch(3);
}

}  // namespace saqg
