// Encode path: CAQEncoder (quantization/caq/caq_encoder.hpp) on the GPU.
//
// The code adjustment is a sequential coordinate descent in FP64 whose every
// accepted move changes the running <o,o_a> and |o_a|^2 read by the next
// dimension (caq_encoder.hpp:57-142); bit-exact codes need the reference's
// exact FP64 operation sequence, so one thread owns one vector and walks its
// dimensions in order.  This file is compiled with --fmad=false: no multiply
// is fused into an add unless written as fma().
#include <cfloat>

#include "device_common.cuh"
#include "saqg_internal.h"

namespace saqg {

namespace {

// Eigen's 16-lane two-accumulator float sum (Redux.h:227-283) in one thread.
template <class F>
__device__ float thread_eigen_sum(int n, F f) {
    const int aligned = n & ~15, aligned2 = n & ~31;
    if (aligned == 0) {
        float r = f(0);
        for (int i = 1; i < n; ++i) r = __fadd_rn(r, f(i));
        return r;
    }
    float r0[16], r1[16];
#pragma unroll
    for (int l = 0; l < 16; ++l) r0[l] = f(l);
    if (aligned > 16) {
#pragma unroll
        for (int l = 0; l < 16; ++l) r1[l] = f(16 + l);
        for (int idx = 32; idx < aligned2; idx += 32)
#pragma unroll
            for (int l = 0; l < 16; ++l) {
                r0[l] = __fadd_rn(r0[l], f(idx + l));
                r1[l] = __fadd_rn(r1[l], f(idx + 16 + l));
            }
#pragma unroll
        for (int l = 0; l < 16; ++l) r0[l] = __fadd_rn(r0[l], r1[l]);
        if (aligned > aligned2)
#pragma unroll
            for (int l = 0; l < 16; ++l) r0[l] = __fadd_rn(r0[l], f(aligned2 + l));
    }
    float x[8], y[4];
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = __fadd_rn(r0[i], r0[i + 8]);
#pragma unroll
    for (int i = 0; i < 4; ++i) y[i] = __fadd_rn(x[i], x[i + 4]);
    float r = __fadd_rn(__fadd_rn(y[0], y[2]), __fadd_rn(y[1], y[3]));
    for (int i = aligned; i < n; ++i) r = __fadd_rn(r, f(i));
    return r;
}

// encode + code_adjustment + encode_and_fac (caq_encoder.hpp:57-247) for one vector.
__device__ void caq_encode_one(const float *__restrict__ o, int D, int bits, const float *__restrict__ cent, int rdlmt,
                               float eps, int32_t *__restrict__ code, float *__restrict__ fac) {
    double v_mx = 0, v_mi = 0, delta = 0, ip = 0, oa2 = 0;
    if (bits > 0) {
        const int cmax = (1 << bits) - 1;
        float mx = o[0], mn = o[0];
        for (int j = 1; j < D; ++j) {
            mx = fmaxf(mx, o[j]);
            mn = fminf(mn, o[j]);
        }
        v_mx = (double)fmaxf(mx, -mn);
        v_mi = -v_mx;
        delta = __ddiv_rn(__dsub_rn(v_mx, v_mi), (double)(cmax + 1));
        const double vec_sum = (double)thread_eigen_sum(D, [&](int i) { return o[i]; });
        double ip_o_code = 0;
        uint64_t code_l2 = 0;
        uint32_t code_sum = 0;
        const float vmi_f = (float)v_mi, d_f = (float)delta;
        for (int j = 0; j < D; ++j) {
            float cf = 0.0f;
            if (delta != 0) cf = fminf(floorf(__fdiv_rn(__fsub_rn(o[j], vmi_f), d_f)), (float)cmax);
            ip_o_code = __dadd_rn(ip_o_code, (double)__fmul_rn(cf, o[j]));
            const int c = (int)cf;
            code[j] = c;
            code_l2 += (uint64_t)(c * c);
            code_sum += (uint32_t)c;
        }
        ip = __dadd_rn(__dmul_rn(ip_o_code, delta), __dmul_rn(__dadd_rn(v_mi, __dmul_rn(0.5, delta)), vec_sum));
        const double dd = __dmul_rn(delta, delta);
        oa2 = __dadd_rn(__dmul_rn(dd, (double)code_l2),
                        __dmul_rn(__dadd_rn(dd, __dmul_rn(__dmul_rn(2.0, delta), v_mi)), (double)code_sum));
        const double k3 = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(0.25, delta), delta), __dmul_rn(delta, v_mi)),
                                    __dmul_rn(v_mi, v_mi));
        oa2 = __dadd_rn(oa2, __dmul_rn(k3, (double)D));
        if (rdlmt && oa2 != 0) {
            const double re_eps = __dmul_rn((double)eps, oa2);
            for (int adj = 1, round = 1; adj; round++) {
                adj = 0;
                for (int j = 0; j < D; ++j) {
                    int cur = 0;
                    const float ov = o[j];
                    double oa = __dadd_rn(__dmul_rn(__dadd_rn((double)code[j], 0.5), delta), v_mi);
                    int c = code[j];
                    const double tmp = __dsub_rn(oa2, __dmul_rn(oa, oa));
                    const double ipd = __dmul_rn(delta, (double)ov);
                    while (c < cmax) {
                        const double nq = __dadd_rn(oa, delta), nl = __dadd_rn(tmp, __dmul_rn(nq, nq)),
                                     ni = __dadd_rn(ip, ipd);
                        if (__dmul_rn(__dadd_rn(__dmul_rn(ip, ip), re_eps), nl) >= __dmul_rn(__dmul_rn(ni, ni), oa2)) break;
                        c++;
                        ip = ni;
                        oa = nq;
                        oa2 = nl;
                        cur++;
                    }
                    while (c > 0) {
                        const double nq = __dsub_rn(oa, delta), nl = __dadd_rn(tmp, __dmul_rn(nq, nq)),
                                     ni = __dsub_rn(ip, ipd);
                        if (__dmul_rn(__dadd_rn(__dmul_rn(ip, ip), re_eps), nl) >= __dmul_rn(__dmul_rn(ni, ni), oa2)) break;
                        c--;
                        ip = ni;
                        oa = nq;
                        oa2 = nl;
                        cur++;
                    }
                    if (code[j] != c) {
                        code[j] = c;
                        adj += cur;
                    }
                }
                if (rdlmt && round >= rdlmt) break;
                double ci = 0, co = 0;
                for (int j = 0; j < D; ++j) {
                    const double qv = __dadd_rn(__dmul_rn(__dadd_rn((double)code[j], 0.5), delta), v_mi);
                    ci = __dadd_rn(ci, __dmul_rn(qv, (double)o[j]));
                    co = __dadd_rn(co, __dmul_rn(qv, qv));
                }
                oa2 = co;
                ip = ci;
            }
        }
    } else {
        for (int j = 0; j < D; ++j) code[j] = 0;
    }
    const double o_l2sqr = (double)thread_eigen_sum(D, [&](int i) { return __fmul_rn(o[i], o[i]); });
    const double o_l2norm = __dsqrt_rn(o_l2sqr);
    double rescale = ip != 0 ? __ddiv_rn(o_l2sqr, ip) : 0.0;
    const double err = __dmul_rn(
        __dmul_rn(o_l2sqr, (double)1.9f),
        __dsqrt_rn(__ddiv_rn(__dsub_rn(__ddiv_rn(__dmul_rn(o_l2sqr, oa2), __dmul_rn(ip, ip)), 1.0), (double)(D - 1))));
    if (v_mx != 0) {
        const double s = __ddiv_rn(1.0, v_mx);
        delta = __dmul_rn(delta, s);
        rescale = __dmul_rn(rescale, v_mx);
        v_mi = __dmul_rn(v_mi, s);
    }
    float ipc = 0.0f;
    if (bits > 1 && cent) {
        const float df = (float)delta, vf = (float)v_mi;
        ipc = thread_eigen_sum(D, [&](int i) { return __fmul_rn(cent[i], __fadd_rn(__fmul_rn((float)code[i], df), vf)); });
    }
    fac[0] = (float)o_l2norm;
    fac[1] = ipc;
    fac[2] = (float)rescale;
    fac[3] = (float)err;
}

__global__ void k_caq_encode(const float *__restrict__ resid, int64_t n, int D, int bits, const float *__restrict__ cent,
                             int rdlmt, float eps, int32_t *__restrict__ codes, float *__restrict__ facs) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    caq_encode_one(resid + v * D, D, bits, cent, rdlmt, eps, codes + v * D, facs + v * 4);
}

}  // namespace

void run_caq_encode(const float *resid, int64_t n, int64_t dim, int bits, const float *cent, int rdlmt, float eps,
                    int32_t *codes, float *facs, int mem, cudaStream_t st) {
    if (n == 0) return;
    const float *dr = resid, *dc = cent;
    int32_t *dcodes = codes;
    float *dfacs = facs;
    void *buf = nullptr;
    if (mem == SAQG_MEM_HOST) {
        const size_t br = 4 * (size_t)n * dim, bc = cent ? 4 * (size_t)dim : 0, bo = 4 * (size_t)n * dim,
                     bf = 16 * (size_t)n;
        SAQG_CUDA_TRY(cudaMalloc(&buf, br + bc + bo + bf + 64));
        char *p = (char *)buf;
        SAQG_CUDA_TRY(cudaMemcpyAsync(p, resid, br, cudaMemcpyHostToDevice, st));
        dr = (const float *)p;
        if (cent) {
            SAQG_CUDA_TRY(cudaMemcpyAsync(p + br, cent, bc, cudaMemcpyHostToDevice, st));
            dc = (const float *)(p + br);
        }
        dcodes = (int32_t *)(p + br + bc);
        dfacs = (float *)(p + br + bc + bo);
    }
    const int tpb = 64;
    k_caq_encode<<<(unsigned)((n + tpb - 1) / tpb), tpb, 0, st>>>(dr, n, (int)dim, bits, dc, rdlmt, eps, dcodes, dfacs);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        if (buf) cudaFree(buf);
        throw Error{SAQG_ERR_CUDA, std::string("k_caq_encode launch failed: ") + cudaGetErrorString(e)};
    }
    count_launch(1);
    if (mem == SAQG_MEM_HOST) {
        SAQG_CUDA_TRY(cudaMemcpyAsync(codes, dcodes, 4 * (size_t)n * dim, cudaMemcpyDeviceToHost, st));
        SAQG_CUDA_TRY(cudaMemcpyAsync(facs, dfacs, 16 * (size_t)n, cudaMemcpyDeviceToHost, st));
        SAQG_CUDA_TRY(cudaStreamSynchronize(st));
        cudaFree(buf);
    }
}

Index *construct_index(const float *, int64_t, int64_t, const float *, int64_t, const uint32_t *,
                       const saqg_quantize_config &, const float *, const float *, uint64_t) {
    throw Error{SAQG_ERR_INVALID, "index construction on the GPU is not available in this build"};
}

}  // namespace saqg
