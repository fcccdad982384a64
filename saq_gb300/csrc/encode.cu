// Encode path: CAQEncoder (quantization/caq/caq_encoder.hpp) on the GPU.
//
// The code adjustment is a sequential coordinate descent in FP64 whose every
// accepted move changes the running <o,o_a> and |o_a|^2 read by the next
// dimension (caq_encoder.hpp:57-142); bit-exact codes need the reference's
// exact FP64 operation sequence, so one thread owns one vector and walks its
// dimensions in order.  In index construction the 32 lanes of a warp encode
// 32 vectors whose residuals and codes are interleaved by dimension, so every
// step of the 32 chains is one coalesced access.  This file is compiled with
// --fmad=false: no multiply is fused into an add unless written as fma().
#include <cfloat>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

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

// encode + code_adjustment + encode_and_fac (caq_encoder.hpp:57-247) for one
// vector whose dimension j lies at o_[j * STR] (its code at code_[j * STR]):
// STR = 1 for a row-major vector, 32 for a vector of a warp-interleaved group,
// where the 32 lanes of a warp encode 32 vectors and every load and store of
// the warp at dimension j is one contiguous 128-byte access.
template <int STR>
__device__ void caq_encode_one(const float *__restrict__ o_, int D, int bits, const float *__restrict__ cent, int rdlmt,
                               float eps, int32_t *__restrict__ code_, float *__restrict__ fac) {
    auto o = [&](int j) { return o_[(int64_t)j * STR]; };
    auto code = [&](int j) -> int32_t & { return code_[(int64_t)j * STR]; };
    double v_mx = 0, v_mi = 0, delta = 0, ip = 0, oa2 = 0;
    if (bits > 0) {
        const int cmax = (1 << bits) - 1;
        float mx = o(0), mn = o(0);
        for (int j = 1; j < D; ++j) {
            mx = fmaxf(mx, o(j));
            mn = fminf(mn, o(j));
        }
        v_mx = (double)fmaxf(mx, -mn);
        v_mi = -v_mx;
        delta = __ddiv_rn(__dsub_rn(v_mx, v_mi), (double)(cmax + 1));
        const double vec_sum = (double)thread_eigen_sum(D, [&](int i) { return o(i); });
        double ip_o_code = 0;
        uint64_t code_l2 = 0;
        uint32_t code_sum = 0;
        const float vmi_f = (float)v_mi, d_f = (float)delta;
        for (int j = 0; j < D; ++j) {
            float cf = 0.0f;
            if (delta != 0) cf = fminf(floorf(__fdiv_rn(__fsub_rn(o(j), vmi_f), d_f)), (float)cmax);
            ip_o_code = __dadd_rn(ip_o_code, (double)__fmul_rn(cf, o(j)));
            const int c = (int)cf;
            code(j) = c;
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
                    const float ov = o(j);
                    double oa = __dadd_rn(__dmul_rn(__dadd_rn((double)code(j), 0.5), delta), v_mi);
                    int c = code(j);
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
                    if (code(j) != c) {
                        code(j) = c;
                        adj += cur;
                    }
                }
                if (rdlmt && round >= rdlmt) break;
                double ci = 0, co = 0;
                for (int j = 0; j < D; ++j) {
                    const double qv = __dadd_rn(__dmul_rn(__dadd_rn((double)code(j), 0.5), delta), v_mi);
                    ci = __dadd_rn(ci, __dmul_rn(qv, (double)o(j)));
                    co = __dadd_rn(co, __dmul_rn(qv, qv));
                }
                oa2 = co;
                ip = ci;
            }
        }
    } else {
        for (int j = 0; j < D; ++j) code(j) = 0;
    }
    const double o_l2sqr = (double)thread_eigen_sum(D, [&](int i) { return __fmul_rn(o(i), o(i)); });
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
        ipc = thread_eigen_sum(D, [&](int i) { return __fmul_rn(cent[i], __fadd_rn(__fmul_rn((float)code(i), df), vf)); });
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
    caq_encode_one<1>(resid + v * D, D, bits, cent, rdlmt, eps, codes + v * D, facs + v * 4);
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

// ---------------------------------------------------------------- construct
namespace {

// SaqDataMaker::compute_variance (saq_data.hpp:95-100): column means by Eigen's
// packetwise reduction (PartialReduxEvaluator.h:102-128), variances of the
// rowwise() difference by a sequential column sum (that expression has no
// packet access); both divided by the row count.  One thread per column.
__global__ void k_colwise_var(const float *__restrict__ x, int64_t n, int D, float *__restrict__ var) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= D) return;
    float p = x[c];
    const int64_t size4 = (n - 1) & ~int64_t(3);
    int64_t i = 1;
    for (; i < size4; i += 4) {
        const float a = __fadd_rn(x[i * D + c], x[(i + 1) * D + c]);
        const float b = __fadd_rn(x[(i + 2) * D + c], x[(i + 3) * D + c]);
        p = __fadd_rn(p, __fadd_rn(a, b));
    }
    for (; i < n; ++i) p = __fadd_rn(p, x[i * D + c]);
    const float mean = __fdiv_rn(p, (float)n);
    float v = 0.0f;
    for (int64_t r = 0; r < n; ++r) {
        const float d = __fsub_rn(x[r * D + c], mean);
        v = r == 0 ? __fmul_rn(d, d) : __fadd_rn(v, __fmul_rn(d, d));
    }
    var[c] = __fdiv_rn(v, (float)n);
}

// Rotated residuals of one segment: out[v][i] = (x_v . P[:, i]) - rc[cid_v][i],
// where x_v is rows[v]'s slice [off, off + dim) of the data, zero-padded past D,
// and the dot product follows Eigen's GEMV order (one FMA chain per block of 16
// inputs, or one chain when dim < 128, blocks added in order).  Tile: 64
// vectors x 64 outputs per CTA, 4 x 4 per thread.
constexpr int kRT = 64, kRK = 16;
__global__ void __launch_bounds__(256) k_rotate(const float *__restrict__ data, int D, const int64_t *__restrict__ rows,
                                                int64_t nv, int off, int dim, const float *__restrict__ P,
                                                const float *__restrict__ rc, const int32_t *__restrict__ cid,
                                                float *__restrict__ out, int interleaved) {
    __shared__ float xs[kRK][kRT + 1];
    __shared__ float ps[kRK][kRT];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int64_t v0 = (int64_t)blockIdx.y * kRT;
    const int o0 = blockIdx.x * kRT;
    const int fold = dim < 128 ? dim : 16;
    float res[4][4], c[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) res[a][b] = c[a][b] = 0.0f;
    for (int j0 = 0; j0 < dim; j0 += kRK) {
        for (int t = threadIdx.x; t < kRT * kRK; t += 256) {
            const int r = t / kRK, k = t % kRK;
            const int64_t v = v0 + r;
            const int gj = off + j0 + k;
            float val = 0.0f;
            if (v < nv && gj < D) val = data[rows[v] * D + gj];
            xs[k][r] = val;
            const int rr = t / kRT, cc = t % kRT;
            ps[rr][cc] = (o0 + cc < dim) ? P[(int64_t)(j0 + rr) * dim + o0 + cc] : 0.0f;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kRK; ++k) {
            float xv[4], pv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) xv[a] = xs[k][ty * 4 + a];
#pragma unroll
            for (int b = 0; b < 4; ++b) pv[b] = ps[k][tx * 4 + b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) c[a][b] = fmaf(pv[b], xv[a], c[a][b]);
        }
        if ((j0 + kRK) % fold == 0) {
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    res[a][b] = fmaf(c[a][b], 1.0f, res[a][b]);
                    c[a][b] = 0.0f;
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int64_t v = v0 + ty * 4 + a;
        if (v >= nv) continue;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int o = o0 + tx * 4 + b;
            if (o >= dim) continue;
            const float r = rc ? __fsub_rn(res[a][b], rc[(int64_t)cid[v] * dim + o]) : res[a][b];
            out[interleaved ? (v >> 5) * (int64_t)dim * 32 + (int64_t)o * 32 + (v & 31) : v * dim + o] = r;
        }
    }
}

// Un-rotated centroid slice (zero-padded) of cluster c, as the reference passes
// it to encode_and_fac for ip_cent_oa (quantizer.hpp:64, saq_quantizer.hpp:51-54).
__global__ void k_centroid_slices(const float *__restrict__ cent, int64_t K, int D, int off, int dim,
                                  float *__restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= K * dim) return;
    const int64_t c = t / dim;
    const int i = (int)(t % dim);
    out[t] = off + i < D ? cent[c * D + off + i] : 0.0f;
}

// CAQEncoder::encode_and_fac for the vectors of a chunk, each with its own
// cluster's un-rotated centroid slice.  Residuals and codes are warp-interleaved
// ([v / 32][dim][v % 32]): lane l of a warp encodes vector 32 w + l, and each
// step of the 32 sequential FP64 chains reads one coalesced line.
__device__ __forceinline__ int64_t inter_at(int64_t v, int D) { return (v >> 5) * (int64_t)D * 32 + (v & 31); }

__global__ void k_caq_encode_clustered(const float *__restrict__ resid, int64_t n, int D, int bits,
                                       const float *__restrict__ cslices, const int32_t *__restrict__ cid, int rdlmt,
                                       float eps, int32_t *__restrict__ codes, float *__restrict__ facs) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    caq_encode_one<32>(resid + inter_at(v, D), D, bits, cslices + (int64_t)cid[v] * D, rdlmt, eps,
                       codes + inter_at(v, D), facs + v * 4);
}

// CodeHelper<B>::compacted_code8/16 (code_helper.hpp) for one vector (code of
// dimension d at v[d * STR]).
template <int STR>
__device__ void pack_bits8_dev(const int32_t *__restrict__ v, int D, int bits, int shift, int mask,
                               uint8_t *__restrict__ y) {
    auto val = [&](int d) { return (uint32_t)((v[(int64_t)d * STR] >> shift) & mask); };
    switch (bits) {
    case 1:
        for (int i = 0; i < D / 8; ++i) {
            uint32_t b = 0;
            for (int j = 0; j < 8; ++j) b |= (val(i * 8 + j) & 1u) << j;
            y[i] = (uint8_t)b;
        }
        break;
    case 2:
    case 3:
        for (int g = 0; g < D / 64; ++g) {
            uint8_t *b = y + g * (bits == 2 ? 16 : 24);
            const int d0 = g * 64;
            for (int r = 0; r < 16; ++r)
                b[r] = (uint8_t)((val(d0 + r) & 3u) | ((val(d0 + 16 + r) & 3u) << 2) | ((val(d0 + 32 + r) & 3u) << 4) |
                                 ((val(d0 + 48 + r) & 3u) << 6));
            if (bits == 3)
                for (int k = 0; k < 8; ++k) {
                    uint32_t t = 0;
                    for (int m = 0; m < 8; ++m) t |= ((val(d0 + 8 * m + k) >> 2) & 1u) << m;
                    b[16 + k] = (uint8_t)t;
                }
        }
        break;
    case 4:
        for (int g = 0; g < D / 32; ++g)
            for (int r = 0; r < 16; ++r)
                y[g * 16 + r] = (uint8_t)((val(g * 32 + r) & 15u) | ((val(g * 32 + 16 + r) & 15u) << 4));
        break;
    case 6:
    case 7:
        for (int g = 0; g < D / 64; ++g) {
            uint8_t *b = y + g * (bits == 6 ? 48 : 56);
            const int d0 = g * 64;
            for (int r = 0; r < 16; ++r) {
                b[r] = (uint8_t)((val(d0 + r) & 63u) | (((val(d0 + 32 + r) >> 4) & 3u) << 6));
                b[16 + r] = (uint8_t)((val(d0 + 16 + r) & 63u) | (((val(d0 + 48 + r) >> 4) & 3u) << 6));
                b[32 + r] = (uint8_t)((val(d0 + 32 + r) & 15u) | ((val(d0 + 48 + r) & 15u) << 4));
            }
            if (bits == 7)
                for (int k = 0; k < 8; ++k) {
                    uint32_t t = 0;
                    for (int m = 0; m < 8; ++m) t |= ((val(d0 + 8 * m + k) >> 6) & 1u) << m;
                    b[48 + k] = (uint8_t)t;
                }
        }
        break;
    case 8:
        for (int d = 0; d < D; ++d) y[d] = (uint8_t)val(d);
        break;
    default:
        break;
    }
}

template <int STR>
__device__ void pack_excode_dev(const int32_t *__restrict__ code, int D, int exb, uint8_t *__restrict__ y) {
    const int lowmask = (1 << exb) - 1;
    if (exb > 8) {  // compacted_code16: low bytes, then the remaining bits in their own layout
        for (int d = 0; d < D; ++d) y[d] = (uint8_t)(code[(int64_t)d * STR] & lowmask & 0xFF);
        const int hb = exb - 8;
        if (hb == 5) {
            pack_bits8_dev<STR>(code, D, 4, 9, 15, y + D);
            pack_bits8_dev<STR>(code, D, 1, 8, 1, y + D + D / 2);
        } else {
            pack_bits8_dev<STR>(code, D, hb, 8, (1 << hb) - 1, y + D);
        }
    } else if (exb == 5) {  // CodeHelper<5>: 4-bit layout of code>>1, then the low bit
        pack_bits8_dev<STR>(code, D, 4, 1, 15, y);
        pack_bits8_dev<STR>(code, D, 1, 0, 1, y + D / 2);
    } else {
        pack_bits8_dev<STR>(code, D, exb, 0, lowmask, y);
    }
}

// ClusterPacker::store_and_pack + finalize_and_store (cluster_packer.hpp:59-116)
// into the device layout (saqg_internal.h): one thread per vector.
__global__ void k_pack(const int32_t *__restrict__ codes, const float *__restrict__ facs, int64_t n, int64_t vbase,
                       const int32_t *__restrict__ cid, const int64_t *__restrict__ blk_off,
                       const int64_t *__restrict__ vec_off, SegDev g) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int64_t gv = vbase + v;
    const int c = cid[v];
    const int64_t pos = gv - vec_off[c];
    const int64_t gb = blk_off[c] + pos / 32;
    const int lane = (int)(pos % 32);
    const float *f = facs + v * 4;
    g.onorm[gb * 32 + lane] = f[0];
    if (g.bits == 0) return;
    g.ipcent[gb * 32 + lane] = f[1];
    g.exfac[gv] = make_float2(f[2], f[3]);
    const int32_t *code = codes + inter_at(v, g.dim);  // warp-interleaved codes: dimension d at code[32 d]
    const int sb = 1 << (g.bits - 1);
    uint8_t *cb = reinterpret_cast<uint8_t *>(g.codes) + (size_t)gb * (g.dim / 8) * 32;
    for (int i = 0; i < g.dim / 8; ++i) {
        uint32_t byte = 0;
        for (int k = 0; k < 8; ++k) byte |= (code[(int64_t)(i * 8 + k) * 32] & sb) ? (0x80u >> k) : 0u;
        cb[((size_t)(i / 8) * 32 + lane) * 8 + (i % 8)] = (uint8_t)byte;
    }
    if (g.bits > 1) pack_excode_dev<32>(code, g.dim, g.bits - 1, g.lcode + (size_t)gv * g.lstride);
}

// Random orthogonal matrix (modified Gram-Schmidt on a Gaussian matrix, FP64,
// seeded) -- the stand-in for Rotator::orthogonalize (rotator.hpp:30-35) when
// the caller gives no rotation.  Returned row-major as P (rows orthonormal).
std::vector<float> random_orthogonal(int64_t d, uint64_t seed) {
    uint64_t st = seed * 0x9E3779B97F4A7C15ull + 0x1234567ull;
    auto next = [&]() {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    auto unif = [&]() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
    std::vector<double> A(d * d);
    for (int64_t i = 0; i < d * d; i += 2) {
        const double u1 = unif(), u2 = unif();
        const double r = std::sqrt(-2.0 * std::log(u1));
        A[i] = r * std::cos(6.283185307179586 * u2);
        if (i + 1 < d * d) A[i + 1] = r * std::sin(6.283185307179586 * u2);
    }
    for (int64_t i = 0; i < d; ++i) {  // rows of A become orthonormal
        double *ri = &A[i * d];
        for (int pass = 0; pass < 2; ++pass)
            for (int64_t k = 0; k < i; ++k) {
                const double *rk = &A[k * d];
                double dot = 0;
                for (int64_t t = 0; t < d; ++t) dot += ri[t] * rk[t];
                for (int64_t t = 0; t < d; ++t) ri[t] -= dot * rk[t];
            }
        double nrm = 0;
        for (int64_t t = 0; t < d; ++t) nrm += ri[t] * ri[t];
        nrm = 1.0 / std::sqrt(nrm);
        for (int64_t t = 0; t < d; ++t) ri[t] *= nrm;
    }
    return std::vector<float>(A.begin(), A.end());
}

void launch_check(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error{SAQG_ERR_CUDA, std::string(what) + " launch failed: " + cudaGetErrorString(e)};
    count_launch(1);
}

struct DevBuf {
    void *p = nullptr;
    explicit DevBuf(size_t bytes) {
        cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
        if (e != cudaSuccess) throw Error{SAQG_ERR_NOMEM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e)};
    }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    template <class T>
    T *as() const {
        return static_cast<T *>(p);
    }
};

}  // namespace

// IVF::construct (index/ivf.hpp:130-184): group by cluster, plan, then per
// segment rotate / encode / pack on the GPU, in chunks of vectors.
Index *construct_index(const float *data, int64_t n, int64_t dim, const float *centroids, int64_t k,
                       const uint32_t *cids, const saqg_quantize_config &cfg, const float *variance,
                       const float *rotations, uint64_t seed, int data_mem) {
    SAQG_REQUIRE(dim % 64 == 0, "dimension must be a multiple of 64 (the reference's load requires it)");
    SAQG_REQUIRE(cfg.avg_bits >= 0 && cfg.avg_bits <= kMaxBits, "avg_bits out of range");
    auto I = std::make_unique<Index>();
    cudaGetDevice(&I->device);
    I->N = n;
    I->D = dim;
    I->K = k;
    // raw config structs as the reference writes them (config.h:12-27)
    uint8_t s20[20] = {0};
    {
        int32_t qt = 0, rd = cfg.caq_adj_rd_lmt, ori = 0;
        std::memcpy(s20, &qt, 4);
        s20[4] = (uint8_t)(cfg.random_rotation != 0);
        s20[5] = 1;
        std::memcpy(s20 + 8, &rd, 4);
        std::memcpy(s20 + 12, &cfg.caq_adj_eps, 4);
        std::memcpy(s20 + 16, &ori, 4);
        int32_t eq = cfg.seg_eqseg;
        std::memcpy(I->qcfg_raw, &cfg.avg_bits, 4);
        std::memcpy(I->qcfg_raw + 4, &eq, 4);
        I->qcfg_raw[8] = (uint8_t)(cfg.enable_segmentation != 0);
        I->qcfg_raw[9] = (uint8_t)(cfg.use_compact_layout != 0);
        std::memcpy(I->qcfg_raw + 12, s20, 20);
    }
    // data on the device
    const float *ddata = data;
    std::unique_ptr<DevBuf> data_buf;
    if (data_mem == SAQG_MEM_HOST) {
        data_buf = std::make_unique<DevBuf>(4 * (size_t)n * dim);
        SAQG_CUDA_TRY(cudaMemcpy(data_buf->p, data, 4 * (size_t)n * dim, cudaMemcpyHostToDevice));
        ddata = data_buf->as<float>();
    }
    // variance
    // variance and the segment plan (the planner runs on the device)
    I->var.resize(dim);
    std::vector<std::pair<int64_t, int64_t>> plan;
    if (variance) {
        std::memcpy(I->var.data(), variance, 4 * dim);
        plan = make_plan_gpu(variance, dim, cfg.avg_bits, cfg.enable_segmentation != 0, cfg.seg_eqseg, false, 0);
    } else {
        DevBuf dv(4 * dim);
        k_colwise_var<<<(unsigned)((dim + 127) / 128), 128>>>(ddata, n, (int)dim, dv.as<float>());
        launch_check("k_colwise_var");
        plan = make_plan_gpu(dv.as<float>(), dim, cfg.avg_bits, cfg.enable_segmentation != 0, cfg.seg_eqseg, true, 0);
        SAQG_CUDA_TRY(cudaMemcpy(I->var.data(), dv.p, 4 * dim, cudaMemcpyDeviceToHost));
    }
    SAQG_REQUIRE(!plan.empty() && plan.size() <= (size_t)kMaxSeg, "planner produced an unsupported plan");
    int64_t roff = 0;
    for (auto &pr : plan) {
        Index::SegHost sg;
        sg.dim = pr.first;
        sg.bits = pr.second;
        std::memcpy(sg.cfg_raw, s20, 20);
        sg.rotated = cfg.random_rotation != 0;
        if (sg.rotated) {
            if (rotations) sg.P.assign(rotations + roff, rotations + roff + sg.dim * sg.dim);
            else sg.P = random_orthogonal(sg.dim, seed + (uint64_t)I->segs.size());
        }
        roff += sg.dim * sg.dim;
        I->segs.push_back(std::move(sg));
    }
    const size_t S = I->segs.size();
    I->compact = S == 1 || cfg.use_compact_layout;
    // group by cluster: ids ascending within each cluster (ivf.hpp:149-157)
    I->sizes.assign(k, 0);
    for (int64_t i = 0; i < n; ++i) {
        SAQG_REQUIRE(cids[i] < (uint64_t)k, "cluster id out of range");
        I->sizes[cids[i]]++;
    }
    I->blk_off.assign(k + 1, 0);
    I->vec_off.assign(k + 1, 0);
    for (int64_t c = 0; c < k; ++c) {
        I->blk_off[c + 1] = I->blk_off[c] + (I->sizes[c] + kBlock - 1) / kBlock;
        I->vec_off[c + 1] = I->vec_off[c] + I->sizes[c];
    }
    const int64_t NB = I->blk_off[k];
    I->total_blocks = NB;
    std::vector<int64_t> rows(n), fill(I->vec_off.begin(), I->vec_off.end() - 1);
    std::vector<int32_t> cid_sorted(n);
    std::vector<uint32_t> ids(n);
    for (int64_t i = 0; i < n; ++i) {
        const int64_t p = fill[cids[i]]++;
        rows[p] = i;
        cid_sorted[p] = (int32_t)cids[i];
        ids[p] = (uint32_t)i;
    }
    // device index arrays
    Index &X = *I;
    DevIndexView &v = X.view;
    float *dcent = (float *)X.dalloc(4 * k * dim);
    X.upload(dcent, centroids, 4 * k * dim);
    v.centroids = dcent;
    {
        float *dvar = (float *)X.dalloc(4 * dim);
        X.upload(dvar, X.var.data(), 4 * dim);
        v.var = dvar;
    }
    uint32_t *dids = (uint32_t *)X.dalloc(4 * n);
    X.upload(dids, ids.data(), 4 * n);
    v.ids = dids;
    int64_t *dbo = (int64_t *)X.dalloc(8 * (k + 1));
    X.upload(dbo, X.blk_off.data(), 8 * (k + 1));
    v.blk_off = dbo;
    int64_t *dvo = (int64_t *)X.dalloc(8 * (k + 1));
    X.upload(dvo, X.vec_off.data(), 8 * (k + 1));
    v.vec_off = dvo;
    DevBuf drows(8 * n), dcid(4 * n);
    SAQG_CUDA_TRY(cudaMemcpy(drows.p, rows.data(), 8 * n, cudaMemcpyHostToDevice));
    SAQG_CUDA_TRY(cudaMemcpy(dcid.p, cid_sorted.data(), 4 * n, cudaMemcpyHostToDevice));
    DevBuf didx(8 * k), dkc(4 * k);
    {
        std::vector<int64_t> ii(k);
        std::vector<int32_t> kc(k);
        for (int64_t c = 0; c < k; ++c) {
            ii[c] = c;
            kc[c] = (int32_t)c;
        }
        SAQG_CUDA_TRY(cudaMemcpy(didx.p, ii.data(), 8 * k, cudaMemcpyHostToDevice));
        SAQG_CUDA_TRY(cudaMemcpy(dkc.p, kc.data(), 4 * k, cudaMemcpyHostToDevice));
    }
    int64_t maxd = 0;
    for (auto &sg : X.segs) maxd = std::max(maxd, sg.dim);
    // chunks of whole 32-vector groups (residuals and codes are warp-interleaved)
    const int64_t chunk = std::max<int64_t>(32, std::min<int64_t>(n, (int64_t)(1u << 30) / (8 * maxd)) / 32 * 32);
    const int64_t chunk_pad = (std::min(chunk, n) + 31) / 32 * 32;
    DevBuf resid(4 * (size_t)chunk_pad * maxd), codes(4 * (size_t)chunk_pad * maxd), facs(16 * (size_t)chunk_pad);
    DevBuf cslice(4 * (size_t)k * maxd);
    int off = 0;
    for (size_t s = 0; s < S; ++s) {
        SegDev &g = v.seg[s];
        const int64_t d = X.segs[s].dim;
        g.dim = (int)d;
        g.bits = (int)X.segs[s].bits;
        g.pv = g.bits ? (int)(d * (g.bits - 1) / 8) : 0;
        g.lstride = (g.pv + 15) / 16 * 16;
        float *dP = nullptr;
        if (X.segs[s].rotated) {
            dP = (float *)X.dalloc(4 * d * d);
            X.upload(dP, X.segs[s].P.data(), 4 * d * d);
        }
        g.P = dP;
        g.codes = (uint2 *)X.dalloc(g.bits ? (size_t)NB * 32 * d / 8 : 0);
        g.onorm = (float *)X.dalloc(4 * (size_t)NB * 32);
        g.ipcent = (float *)X.dalloc(4 * (size_t)NB * 32);
        g.lcode = (uint8_t *)X.dalloc((size_t)n * g.lstride);
        g.exfac = (float2 *)X.dalloc(8 * (size_t)n);
        g.cent = (float *)X.dalloc(4 * (size_t)k * d);
        SAQG_CUDA_TRY(cudaMemset(g.codes, 0, g.bits ? (size_t)NB * 32 * d / 8 : 0));
        SAQG_CUDA_TRY(cudaMemset(g.onorm, 0, 4 * (size_t)NB * 32));
        SAQG_CUDA_TRY(cudaMemset(g.ipcent, 0, 4 * (size_t)NB * 32));
        SAQG_CUDA_TRY(cudaMemset(g.lcode, 0, (size_t)n * g.lstride));
        SAQG_CUDA_TRY(cudaMemset(g.exfac, 0, 8 * (size_t)n));
        // rotated centroids: clus.centroid() = centroid * P (quantizer.hpp:46)
        {
            dim3 grid((unsigned)((d + kRT - 1) / kRT), (unsigned)((k + kRT - 1) / kRT));
            if (dP) {
                k_rotate<<<grid, 256>>>(dcent, (int)dim, didx.as<int64_t>(), k, off, (int)d, dP, nullptr, nullptr, g.cent,
                                        0);
                launch_check("k_rotate(centroids)");
            }
            k_centroid_slices<<<(unsigned)((k * d + 255) / 256), 256>>>(dcent, k, (int)dim, off, (int)d,
                                                                       cslice.as<float>());
            launch_check("k_centroid_slices");
            if (!dP) SAQG_CUDA_TRY(cudaMemcpy(g.cent, cslice.p, 4 * (size_t)k * d, cudaMemcpyDeviceToDevice));
        }
        std::vector<float> ident;
        DevBuf *idP = nullptr;
        std::unique_ptr<DevBuf> idbuf;
        if (!dP) {  // no rotation: residual = x - c, same kernel with an identity matrix
            ident.assign(d * d, 0.0f);
            for (int64_t i = 0; i < d; ++i) ident[i * d + i] = 1.0f;
            idbuf = std::make_unique<DevBuf>(4 * d * d);
            SAQG_CUDA_TRY(cudaMemcpy(idbuf->p, ident.data(), 4 * d * d, cudaMemcpyHostToDevice));
            idP = idbuf.get();
        }
        for (int64_t v0 = 0; v0 < n; v0 += chunk) {
            const int64_t nv = std::min(chunk, n - v0);
            dim3 grid((unsigned)((d + kRT - 1) / kRT), (unsigned)((nv + kRT - 1) / kRT));
            k_rotate<<<grid, 256>>>(ddata, (int)dim, drows.as<int64_t>() + v0, nv, off, (int)d,
                                    dP ? dP : idP->as<float>(), g.cent, dcid.as<int32_t>() + v0, resid.as<float>(), 1);
            launch_check("k_rotate");
            k_caq_encode_clustered<<<(unsigned)((nv + 63) / 64), 64>>>(
                resid.as<float>(), nv, (int)d, g.bits, cslice.as<float>(), dcid.as<int32_t>() + v0, cfg.caq_adj_rd_lmt,
                cfg.caq_adj_eps, codes.as<int32_t>(), facs.as<float>());
            launch_check("k_caq_encode");
            k_pack<<<(unsigned)((nv + 127) / 128), 128>>>(codes.as<int32_t>(), facs.as<float>(), nv, v0,
                                                          dcid.as<int32_t>() + v0, dbo, dvo, g);
            launch_check("k_pack");
        }
        SAQG_CUDA_TRY(cudaDeviceSynchronize());
        off += (int)d;
    }
    finalize_view(X);
    return I.release();
}

}  // namespace saqg
