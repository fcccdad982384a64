// Segment bit planner on the device: SaqDataMaker::dynamic_programming
// (quantization/saq_data.hpp:147-227).
//
// The reference's dynamic program pushes every state f[ns][i][bits] (least sum
// over ns segments of var_sum / 2^b covering the first i 64-dim blocks with
// `bits` total bits) forward to f[ns + 1][i + j][bits + b * 64 j + 64], keeping
// the first strict improvement in its visit order (ns, i, bits, then j, b),
// plus a 0-bit tail segment to the end.  Here each level ns + 1 is computed
// from level ns by one thread per target state (i', B'), which pulls its
// candidates in exactly the order the pushes would reach it: sources by i
// ascending, and for one i by bits ascending, i.e. b descending, the 0-bit tail
// (when i' is the end) last.  The same strict comparisons on the same double
// values give the same table, so the answer and the backtracked plan are the
// reference's.  The answer scan (the 1 % rule) and the backtrack are sequential
// and run in one thread.
#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <string>
#include <vector>

#include "saqg_internal.h"

namespace saqg {

namespace {

constexpr double kLim = DBL_MAX;  // the reference's valid_lmt (numeric_limits<double>::max())

// Sum of one 64-float block in Eigen's 16-lane order (Redux.h:227-283):
// accumulators over packets {0, 2} and {1, 3}, then the 16 -> 1 tree.
__device__ float block_sum64(const float *x) {
    float r0[16];
#pragma unroll
    for (int l = 0; l < 16; ++l) {
        const float a = __fadd_rn(x[l], x[32 + l]);
        const float b = __fadd_rn(x[16 + l], x[48 + l]);
        r0[l] = __fadd_rn(a, b);
    }
    float a[8], b[4];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = __fadd_rn(r0[i], r0[i + 8]);
#pragma unroll
    for (int i = 0; i < 4; ++i) b[i] = __fadd_rn(a[i], a[i + 4]);
    return __fadd_rn(__fadd_rn(b[0], b[2]), __fadd_rn(b[1], b[3]));
}

// vsum[i * H + j] = sum of blocks i .. i + j - 1, accumulated in double from
// block i upward (the reference's var_sum for source i and length j).
__global__ void k_plan_vsum(const float *__restrict__ var, int i_end, int H, double *__restrict__ vsum) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= i_end) return;
    double s = 0.0;
    vsum[(size_t)i * H] = 0.0;
    for (int j = 1; i + j <= i_end; ++j) {
        s = __dadd_rn(s, (double)block_sum64(var + 64 * (size_t)(i + j - 1)));
        vsum[(size_t)i * H + j] = s;
    }
}

__global__ void k_plan_init(double *__restrict__ fv, uint32_t *__restrict__ fs, size_t total) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        fv[t] = t == 0 ? 0.0 : kLim;  // f[0][0][0] = 0
        fs[t] = 0;
    }
}

// Level ns + 1 from level ns (prev / next are one level's H x W slices).
__global__ void k_plan_level(const double *__restrict__ prev, double *__restrict__ next, uint32_t *__restrict__ fs_next,
                             const double *__restrict__ vsum, int i_end, int H, int W, int nbf, int max_bits) {
    const int Bp = blockIdx.x * blockDim.x + threadIdx.x;
    const int ip = blockIdx.y + 1;
    if (Bp >= W || ip > i_end) return;
    double val = kLim;
    uint32_t arg = 0;
    for (int i = 0; i < ip; ++i) {
        const int j = ip - i;
        const double vs = vsum[(size_t)i * H + j];
        for (int b = max_bits; b >= 1; --b) {
            const long long ub = (long long)Bp - (long long)b * j * 64 - nbf;
            if (ub < 0) continue;
            const double cur = prev[(size_t)i * W + ub];
            if (!(cur < kLim)) continue;
            const double cand = __dadd_rn(cur, __ddiv_rn(vs, (double)(1 << b)));
            if (val > cand) {
                val = cand;
                arg = ((uint32_t)i << 4) + (uint32_t)b;
            }
        }
        if (ip == i_end) {  // the 0-bit tail segment from source (i, Bp)
            const double cur = prev[(size_t)i * W + Bp];
            if (cur < kLim) {
                const double cand = __dadd_rn(cur, vs);
                if (cand < val) {
                    val = cand;
                    arg = (uint32_t)i << 4;
                }
            }
        }
    }
    next[(size_t)ip * W + Bp] = val;
    fs_next[(size_t)ip * W + Bp] = arg;
}

// The answer (first end state, in (ns, bits) order, that beats the current one
// by 1 %) and the backtrack; out[0] = number of segments, then (length, bits).
__global__ void k_plan_answer(const double *__restrict__ fv, const uint32_t *__restrict__ fs, int max_ns, int i_end,
                              int H, int W, int tot_bits, int nbf, long long *__restrict__ out, int cap) {
    if (threadIdx.x || blockIdx.x) return;
    auto at = [&](int ns, int i, int b) { return ((size_t)ns * H + i) * W + b; };
    int ans_ns = 0, ans_b = tot_bits;
    for (int ns = 0; ns <= max_ns; ++ns)
        for (int ub = 0; ub <= tot_bits; ++ub) {
            const double cur = fv[at(ns, i_end, ub)];
            if (!(cur < kLim)) continue;
            if (__dmul_rn(cur, 1.01) < fv[at(ans_ns, i_end, ans_b)]) {
                ans_ns = ns;
                ans_b = ub;
            }
        }
    int ns = ans_ns, i = i_end, B = ans_b, n = 0;
    long long tmp[2 * 64];
    // (as the reference: with no segment possible the walk reads the table's
    // untouched state and yields one 0-bit segment; a corrupt table ends the
    // walk with out[0] = -1)
    while (i > 0 && n < 64 && ns >= 0 && B >= 0) {
        const uint32_t s = fs[at(ns, i, B)];
        const int pi = (int)(s >> 4), bits = (int)(s & 0xf);
        if (pi >= i) break;
        const int len = (i - pi) * 64;
        tmp[2 * n] = len;
        tmp[2 * n + 1] = bits;
        ++n;
        --ns;
        i = pi;
        if (bits) B -= bits * len + nbf;
    }
    out[0] = i == 0 ? n : -1;
    for (int k = 0; k < n && k < cap; ++k) {  // reversed: first segment first
        out[1 + 2 * k] = tmp[2 * (n - 1 - k)];
        out[2 + 2 * k] = tmp[2 * (n - 1 - k) + 1];
    }
}

struct DevMem {
    void *p = nullptr;
    explicit DevMem(size_t b) {
        const cudaError_t e = cudaMalloc(&p, b ? b : 16);
        if (e != cudaSuccess) throw Error{SAQG_ERR_NOMEM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e)};
    }
    ~DevMem() {
        if (p) cudaFree(p);
    }
};

void launched(const char *what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error{SAQG_ERR_CUDA, std::string(what) + " launch failed: " + cudaGetErrorString(e)};
    count_launch(1);
}

}  // namespace

// The DP plan from a device-resident variance (dim_padded floats), on `st`.
std::vector<std::pair<int64_t, int64_t>> make_plan_device(const float *dvar, int64_t Dp, float avg_bits,
                                                          cudaStream_t st) {
    SAQG_REQUIRE(Dp > 0 && Dp % 64 == 0, "dim_padded must be a positive multiple of 64");
    const int nbf = 2 * (int)sizeof(float) * 8;
    const int tot_bits = (int)(size_t)(avg_bits * (float)Dp + (float)nbf);
    const int i_end = (int)(Dp / 64), H = i_end + 1, W = tot_bits + 1;
    const int max_ns = avg_bits < 2 ? i_end : i_end / 2;
    const size_t level = (size_t)H * W, total = (size_t)(max_ns + 1) * level;
    DevMem fv(8 * total), fs(4 * total), vs(8 * (size_t)H * H), out(8 * (1 + 2 * 64));
    double *dfv = static_cast<double *>(fv.p);
    uint32_t *dfs = static_cast<uint32_t *>(fs.p);
    double *dvs = static_cast<double *>(vs.p);
    long long *dout = static_cast<long long *>(out.p);
    k_plan_vsum<<<(i_end + 63) / 64, 64, 0, st>>>(dvar, i_end, H, dvs);
    launched("k_plan_vsum");
    k_plan_init<<<(unsigned)std::min<size_t>((total + 255) / 256, 4096), 256, 0, st>>>(dfv, dfs, total);
    launched("k_plan_init");
    for (int ns = 0; ns < max_ns; ++ns) {
        k_plan_level<<<dim3((unsigned)((W + 127) / 128), (unsigned)i_end), 128, 0, st>>>(
            dfv + ns * level, dfv + (ns + 1) * level, dfs + (ns + 1) * level, dvs, i_end, H, W, nbf, kMaxBits);
        launched("k_plan_level");
    }
    k_plan_answer<<<1, 1, 0, st>>>(dfv, dfs, max_ns, i_end, H, W, tot_bits, nbf, dout, 64);
    launched("k_plan_answer");
    long long h[1 + 2 * 64];
    SAQG_CUDA_TRY(cudaMemcpyAsync(h, dout, sizeof(h), cudaMemcpyDeviceToHost, st));
    SAQG_CUDA_TRY(cudaStreamSynchronize(st));
    SAQG_REQUIRE(h[0] >= 1 && h[0] <= 64, "device planner produced no valid plan");
    std::vector<std::pair<int64_t, int64_t>> plan;
    for (long long k = 0; k < h[0]; ++k) plan.emplace_back((int64_t)h[1 + 2 * k], (int64_t)h[2 + 2 * k]);
    return plan;
}

// Equal segmentation needs no program; the DP runs on the device.
std::vector<std::pair<int64_t, int64_t>> make_plan_gpu(const float *var, int64_t Dp, float avg_bits, bool seg,
                                                       int eqseg, bool var_on_device, cudaStream_t st) {
    if (!seg || eqseg > 0) return make_plan(nullptr, Dp, avg_bits, seg, eqseg);
    if (var_on_device) return make_plan_device(var, Dp, avg_bits, st);
    DevMem dv(4 * (size_t)Dp);
    SAQG_CUDA_TRY(cudaMemcpyAsync(dv.p, var, 4 * (size_t)Dp, cudaMemcpyHostToDevice, st));
    return make_plan_device(static_cast<const float *>(dv.p), Dp, avg_bits, st);
}

}  // namespace saqg
