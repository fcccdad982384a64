// Inner products of a query batch with every centroid on the tensor cores:
// ip[q][c] = sum_d Q[q][d] C[c][d] with BF16 operands (rounded to nearest) and
// FP32 accumulation, the first step of the batched centroid ranking
// (FlatInitializer::centroids_distances, initializer.hpp:52-76, for a batch).
// k_probe_shortlist turns each product into a distance interval that provably
// holds the reference's float distance, so the ranking stays exact.  BF16 halves
// the operand bytes that every tile streams from L2 (the bound of this GEMM at
// these shapes) against TF32, for a four times wider interval.
//
// k_probe_gemm is persistent, one CTA of 192 threads per SM, over 128 x 256
// output tiles (queries x centroids), tiles taken round-robin:
//   warp 0 (one thread)  TMA: per 64-dim stage the 128-row query tile and the
//                        256-row centroid tile (BF16, 128-byte swizzle) into a
//                        4-stage ring (48 KB per stage)
//   warp 1 (one thread)  tcgen05.mma kind::f16 (BF16; M = 128, N = 256, K = 16
//                        per instruction) into one of two TMEM accumulators of
//                        256 columns; commits free a stage / publish an
//                        accumulator; warp 1 also owns the 512 TMEM columns
//   warps 2-5            epilogue: tcgen05.ld of their 32 lanes (query rows),
//                        row-major FP32 stores of the products
// Tile t uses accumulator t & 1, so the MMAs of the next tile overlap the
// epilogue of this one.  Every wait is bounded: on a timeout the CTA records
// the error, drains its copies and MMAs, frees TMEM and returns, and the host
// call fails with SAQG_ERR_INTERNAL.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "saqg_internal.h"
#include "tcgen05.cuh"

namespace saqg {

namespace {

using namespace tc;

constexpr int kGmBM = 128;                 // queries per tile (the MMA's M)
constexpr int kGmBN = 256;                 // centroids per tile (the MMA's N)
constexpr int kGmBK = 64;                  // dims per stage: one 128-byte BF16 row
constexpr int kGmStages = 4;
constexpr int kGmThreads = 192;
constexpr int kGmStageA = kGmBM * 128;     // 16 KB
constexpr int kGmStageB = kGmBN * 128;     // 32 KB
constexpr int kGmCols = 512;               // two accumulators of 256 FP32 columns

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M = 128, N = 256.
__device__ __forceinline__ uint32_t idesc_gemm() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kGmBN >> 3) << 17) | ((uint32_t)(kGmBM >> 4) << 24);
}

// x (n floats) -> BF16, rounded to nearest even.
__global__ void k_to_bf16(const float *__restrict__ x, int64_t n, __nv_bfloat16 *__restrict__ y) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16_rn(x[i]);
}

struct GemmArgs {
    int M, N, Kd;       // queries, centroids, dimension
    int tiles_m, tiles_n;
    float *out;         // [M][ldo]
    long long ldo;
    int *err;
};

__global__ void __launch_bounds__(kGmThreads, 1) k_probe_gemm(const __grid_constant__ CUtensorMap tmQ,
                                                             const __grid_constant__ CUtensorMap tmC, GemmArgs g) {
    extern __shared__ uint8_t gm_smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int kch = (g.Kd + kGmBK - 1) / kGmBK, ntiles = g.tiles_m * g.tiles_n;
    const uint32_t raw = smem_u32(gm_smem);
    const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
    uint8_t *sm = gm_smem + pad;
    const uint32_t sA = raw + pad, sB = sA + kGmStages * kGmStageA;
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + kGmStages * (kGmStageA + kGmStageB));
    const uint32_t b0 = smem_u32(bars);
    auto full = [&](int st) { return b0 + 8u * st; };
    auto empty = [&](int st) { return b0 + 8u * (kGmStages + st); };
    auto accf = [&](int i) { return b0 + 8u * (2 * kGmStages + i); };
    auto acce = [&](int i) { return b0 + 8u * (2 * kGmStages + 2 + i); };
    const uint32_t done = b0 + 8u * (2 * kGmStages + 4);
    int *misc = reinterpret_cast<int *>(bars + 2 * kGmStages + 5);  // [0] TMEM address, [1] abort
    volatile int *abort = misc + 1;

    if (tid == 0) {
        for (int st = 0; st < kGmStages; ++st) {
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
                     "r"(kGmCols)
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
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                const int mt = t % g.tiles_m, nt = t / g.tiles_m;
                for (int kc = 0; kc < kch; ++kc, ++it) {
                    const int st = it % kGmStages;
                    const uint32_t ph = (uint32_t)(it / kGmStages) & 1u;
                    if (!mbar_wait(empty(st), ph ^ 1u, abort)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(full(st), kGmStageA + kGmStageB);
                    tma_load_2d(sA + st * kGmStageA, &tmQ, full(st), kc * kGmBK, mt * kGmBM);
                    tma_load_2d(sB + st * kGmStageB, &tmC, full(st), kc * kGmBK, nt * kGmBN);
                }
            }
            if (!ok) {
                atomicExch(g.err, 1);
                for (int k = max(0, it - kGmStages); k < it; ++k)  // copies possibly in flight
                    mbar_drain(full(k % kGmStages), (uint32_t)(k / kGmStages) & 1u);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        // ---- MMA issuer
        if (lane == 0) {
            int it = 0, lt = 0;
            bool ok = true;
            const uint32_t idesc = idesc_gemm();
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++lt) {
                const int buf = lt & 1;
                if (!mbar_wait(acce(buf), (((uint32_t)lt >> 1) & 1u) ^ 1u, abort)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t dacc = tmem + (uint32_t)(buf * kGmBN);
                for (int kc = 0; kc < kch; ++kc, ++it) {
                    const int st = it % kGmStages;
                    const uint32_t ph = (uint32_t)(it / kGmStages) & 1u;
                    if (!mbar_wait(full(st), ph, abort)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint64_t da = sw128_desc(sA + st * kGmStageA), db = sw128_desc(sB + st * kGmStageB);
#pragma unroll
                    for (int kk = 0; kk < kGmBK / 16; ++kk)  // 16 BF16 = 32 bytes per instruction
                        mma_bf16(dacc, da + 2 * kk, db + 2 * kk, idesc, (kc == 0 && kk == 0) ? 0u : 1u);
                    mma_commit(empty(st));
                }
                if (ok) mma_commit(accf(buf));
            }
            if (!ok) atomicExch(g.err, 1);
            mma_commit(done);  // every MMA issued has finished once `done` completes
            mbar_drain(done, 0);
        }
        __syncwarp();
    } else {
        // ---- epilogue: warps 2-5, TMEM lanes (warp % 4) * 32 + lane = query rows of the tile
        const int qt = warp & 3, r = qt * 32 + lane;
        int lt = 0;
        bool ok = true;
        for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++lt) {
            const int mt = t % g.tiles_m, nt = t / g.tiles_m;
            const int buf = lt & 1;
            if (ok && !mbar_wait(accf(buf), ((uint32_t)lt >> 1) & 1u, abort)) ok = false;
            tc_fence_after();
            if (!__all_sync(kFullMask, ok)) {
                ok = false;
                break;
            }
            const int row = mt * kGmBM + r, c0 = nt * kGmBN;
            float *orow = g.out + (long long)row * g.ldo + c0;
            const bool vec = row < g.M && c0 + kGmBN <= g.N && (g.ldo & 3) == 0;
            for (int n0 = 0; n0 < kGmBN; n0 += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(qt * 32) << 16) + (uint32_t)(buf * kGmBN + n0), v);
                if (vec) {
                    float4 *o4 = reinterpret_cast<float4 *>(orow + n0);
#pragma unroll
                    for (int i = 0; i < 4; ++i) o4[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
                } else if (row < g.M) {
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        if (c0 + n0 + i < g.N) orow[n0 + i] = v[i];
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(acce(buf));
        }
        if (!ok && lane == 0) atomicExch(g.err, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kGmCols) : "memory");
    }
}

constexpr size_t gemm_smem() {
    return 1024 + (size_t)kGmStages * (kGmStageA + kGmStageB) + 8 * (2 * kGmStages + 5) + 16;
}

PFN_cuTensorMapEncodeTiled_v12000 map_encoder() {
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

// Row-major BF16 matrix [rows][cols] read in (64 x box_rows) boxes, 128-byte swizzle.
CUtensorMap bf16_map(const __nv_bfloat16 *base, int64_t cols, int64_t rows, int box_rows) {
    CUtensorMap m;
    const cuuint64_t gdim[2] = {(cuuint64_t)cols, (cuuint64_t)std::max<int64_t>(rows, 1)};
    const cuuint64_t gstride[1] = {(cuuint64_t)cols * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kGmBK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = map_encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16 *>(base), gdim, gstride,
                                     box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error{SAQG_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r)};
    return m;
}

int sms() {
    static int n = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
    });
    return n;
}

}  // namespace

void to_bf16(const float *x, int64_t n, void *y, cudaStream_t st) {
    if (n <= 0) return;
    const unsigned grid = (unsigned)std::min<int64_t>((n + 255) / 256, 4 * (int64_t)sms() * 8);
    k_to_bf16<<<grid, 256, 0, st>>>(x, n, static_cast<__nv_bfloat16 *>(y));
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error{SAQG_ERR_CUDA, std::string("k_to_bf16 launch failed: ") + cudaGetErrorString(e)};
    count_launch(1);
}

void probe_ip_gemm(const void *q_bf16, int64_t nq, const void *cent_bf16, int64_t K, int64_t D, float *ip, int *err,
                   cudaStream_t st) {
    SAQG_REQUIRE(D % 8 == 0 && D > 0, "the probe GEMM needs a dimension that is a multiple of 8");
    SAQG_REQUIRE(nq < (int64_t)1 << 31 && K < (int64_t)1 << 31, "probe GEMM too large");
    SAQG_REQUIRE(((uintptr_t)q_bf16 & 15) == 0 && ((uintptr_t)cent_bf16 & 15) == 0,
                 "probe GEMM operands must be 16-byte aligned");
    if (nq == 0 || K == 0) return;
    const CUtensorMap tmQ = bf16_map(static_cast<const __nv_bfloat16 *>(q_bf16), D, nq, kGmBM);
    const CUtensorMap tmC = bf16_map(static_cast<const __nv_bfloat16 *>(cent_bf16), D, K, kGmBN);
    GemmArgs g;
    g.M = (int)nq;
    g.N = (int)K;
    g.Kd = (int)D;
    g.tiles_m = (int)((nq + kGmBM - 1) / kGmBM);
    g.tiles_n = (int)((K + kGmBN - 1) / kGmBN);
    g.out = ip;
    g.ldo = K;
    g.err = err;
    SAQG_CUDA_TRY(cudaFuncSetAttribute(k_probe_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem()));
    const int64_t ntiles = (int64_t)g.tiles_m * g.tiles_n;
    const unsigned grid = (unsigned)std::min<int64_t>(ntiles, sms());
    k_probe_gemm<<<grid, kGmThreads, gemm_smem(), st>>>(tmQ, tmC, g);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error{SAQG_ERR_CUDA, std::string("k_probe_gemm launch failed: ") + cudaGetErrorString(e)};
    count_launch(1);
}

}  // namespace saqg
