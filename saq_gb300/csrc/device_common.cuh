// Device primitives that reproduce the reference's floating-point order.
//
// The reference (saqlib/, compiled with -O3 -march=native -ffp-contract=off on
// an AVX-512 host) evaluates its float reductions in fixed SIMD orders.  A
// 32-lane warp maps onto them directly:
//   * Eigen's vectorised sum (Eigen/src/Core/Redux.h:227-283): two 16-lane
//     accumulators take the even and odd 16-float packets; lanes 0-15 of the
//     warp hold accumulator 0, lanes 16-31 accumulator 1.
//   * predux<Packet16f> and GCC's _mm512_reduce_add_ps: lane i + lane i+8,
//     then +4, +2, +1 -- exactly a 16-wide shfl_down tree.
//   * _mm512_reduce_min_ps(_mm512_min_ps(a, b)): the same tree with x86
//     min semantics ((a < b) ? a : b, second operand on NaN).
// This translation unit is compiled with --fmad=false; every FMA below is an
// explicit fmaf(), matching the reference's explicit _mm512_fmadd_ps calls.
#pragma once

#include <cstdint>

namespace saqg {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float minps(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float maxps(float a, float b) { return a > b ? a : b; }

// Eigen redux over n elements, one warp.  f(i) yields element i (already
// rounded on its own).  Result returned to every lane.
template <class F>
__device__ __forceinline__ float warp_eigen_sum(int n, F f) {
    const int lane = threadIdx.x & 31, l = lane & 15, half = lane >> 4;
    const int aligned = n & ~15, aligned2 = n & ~31;
    float r;
    if (aligned == 0) {
        r = 0.0f;
        if (lane == 0 && n > 0) {
            r = f(0);
            for (int i = 1; i < n; ++i) r = __fadd_rn(r, f(i));
        }
        return __shfl_sync(kFull, r, 0);
    }
    float acc;
    if (aligned > 16) {
        acc = f(16 * half + l);
        for (int p = half + 2; p < aligned2 / 16; p += 2) acc = __fadd_rn(acc, f(16 * p + l));
        const float other = __shfl_down_sync(kFull, acc, 16);
        acc = __fadd_rn(acc, other);
        if (aligned > aligned2 && lane < 16) acc = __fadd_rn(acc, f(aligned2 + l));
    } else {
        acc = lane < 16 ? f(l) : 0.0f;
    }
    acc = __fadd_rn(acc, __shfl_down_sync(kFull, acc, 8));
    acc = __fadd_rn(acc, __shfl_down_sync(kFull, acc, 4));
    acc = __fadd_rn(acc, __shfl_down_sync(kFull, acc, 2));
    acc = __fadd_rn(acc, __shfl_down_sync(kFull, acc, 1));
    r = acc;
    if (lane == 0)
        for (int i = aligned; i < n; ++i) r = __fadd_rn(r, f(i));
    return __shfl_sync(kFull, r, 0);
}

// 16-lane add tree inside a half-warp (lane l of the half holds lane l of the
// SIMD accumulator).  Result valid in the half's lane 0.
__device__ __forceinline__ float half_reduce16(float v, unsigned mask) {
    v = __fadd_rn(v, __shfl_down_sync(mask, v, 8, 16));
    v = __fadd_rn(v, __shfl_down_sync(mask, v, 4, 16));
    v = __fadd_rn(v, __shfl_down_sync(mask, v, 2, 16));
    v = __fadd_rn(v, __shfl_down_sync(mask, v, 1, 16));
    return v;
}

// _mm512_reduce_min_ps(_mm512_min_ps(d[0..15], d[16..31])) with lane j holding d[j].
__device__ __forceinline__ float warp_min_tree(float x) {
    float v = minps(x, __shfl_down_sync(kFull, x, 16));  // (a < b) ? a : b, a = lanes 0-15
    float o = __shfl_down_sync(kFull, v, 8);
    v = minps(o, v);                                     // T3 = min(upper, lower)
    o = __shfl_down_sync(kFull, v, 4);
    v = minps(o, v);                                     // T6
    o = __shfl_down_sync(kFull, v, 2);
    v = minps(v, o);                                     // T8 = min(T6, shuffled)
    o = __shfl_down_sync(kFull, v, 1);
    v = minps(v, o);                                     // T10
    return __shfl_sync(kFull, v, 0);
}

// --------------------------------------------------------------- ex-codes
// One 16-lane chain of CodeHelper<B>::compute_ip, lane l of a half-warp
// accumulating dims l, l+16, l+32, ... in increasing order.  The reference's
// compacted layouts were designed for 16-lane SIMD, so lane l reads the same
// byte positions in every group of dims; the chains read them straight from
// global memory (L1/L2), 16 consecutive bytes per half-warp load.
template <int B>
__device__ __forceinline__ float chain_bits(const float *__restrict__ q, const uint8_t *__restrict__ y, int D, int l);

template <>
__device__ __forceinline__ float chain_bits<1>(const float *__restrict__ q, const uint8_t *__restrict__ y, int D, int l) {
    // CodeHelper<1>: bit d of the little-endian bit string; masked adds
    float acc = 0.0f;
    for (int g = 0; g < D; g += 16) {
        const uint32_t m = (uint32_t)y[g / 8] | ((uint32_t)y[g / 8 + 1] << 8);
        acc = __fadd_rn(acc, ((m >> l) & 1u) ? q[g + l] : 0.0f);
    }
    return acc;
}

template <>
__device__ __forceinline__ float chain_bits<2>(const float *__restrict__ q, const uint8_t *__restrict__ y, int D, int l) {
    float acc = 0.0f;
    for (int g = 0; g < D; g += 64) {
        const uint32_t b = y[(g / 64) * 16 + l];
#pragma unroll
        for (int k = 0; k < 4; ++k) acc = fmaf((float)((b >> (2 * k)) & 3u), q[g + 16 * k + l], acc);
    }
    return acc;
}

template <>
__device__ __forceinline__ float chain_bits<3>(const float *__restrict__ q, const uint8_t *__restrict__ y, int D, int l) {
    float acc = 0.0f;
    for (int g = 0; g < D; g += 64) {
        const uint8_t *gp = y + (g / 64) * 24;
        const uint32_t b = gp[l];
        // top bit of dim (16k + l) sits in byte 16 + (l & 7), bit 2k + (l >> 3)
        const uint32_t t = gp[16 + (l & 7)];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t v = ((b >> (2 * k)) & 3u) | (((t >> (2 * k + (l >> 3))) & 1u) << 2);
            acc = fmaf((float)v, q[g + 16 * k + l], acc);
        }
    }
    return acc;
}

template <>
__device__ __forceinline__ float chain_bits<4>(const float *__restrict__ q, const uint8_t *__restrict__ y, int D, int l) {
    float acc = 0.0f;
    for (int g = 0; g < D; g += 32) {
        const uint32_t b = y[(g / 32) * 16 + l];
        acc = fmaf((float)(b & 15u), q[g + l], acc);
        acc = fmaf((float)(b >> 4), q[g + 16 + l], acc);
    }
    return acc;
}

template <int B>  // 6 or 7
__device__ __forceinline__ float chain_67(const float *__restrict__ q, const uint8_t *__restrict__ y, int D, int l) {
    float acc = 0.0f;
    for (int g = 0; g < D; g += 64) {
        const uint8_t *gp = y + (g / 64) * (B == 6 ? 48 : 56);
        const uint32_t b0 = gp[l], b1 = gp[16 + l], b2 = gp[32 + l];
        uint32_t v0 = b0 & 63u, v1 = b1 & 63u;
        uint32_t v2 = ((b0 >> 6) << 4) | (b2 & 15u), v3 = ((b1 >> 6) << 4) | (b2 >> 4);
        if (B == 7) {
            const uint32_t t = gp[48 + (l & 7)];
            const int sh = l >> 3;
            v0 |= ((t >> (0 + sh)) & 1u) << 6;
            v1 |= ((t >> (2 + sh)) & 1u) << 6;
            v2 |= ((t >> (4 + sh)) & 1u) << 6;
            v3 |= ((t >> (6 + sh)) & 1u) << 6;
        }
        acc = fmaf((float)v0, q[g + l], acc);
        acc = fmaf((float)v1, q[g + 16 + l], acc);
        acc = fmaf((float)v2, q[g + 32 + l], acc);
        acc = fmaf((float)v3, q[g + 48 + l], acc);
    }
    return acc;
}

template <>
__device__ __forceinline__ float chain_bits<6>(const float *__restrict__ q, const uint8_t *__restrict__ y, int D, int l) {
    return chain_67<6>(q, y, D, l);
}
template <>
__device__ __forceinline__ float chain_bits<7>(const float *__restrict__ q, const uint8_t *__restrict__ y, int D, int l) {
    return chain_67<7>(q, y, D, l);
}

template <>
__device__ __forceinline__ float chain_bits<8>(const float *__restrict__ q, const uint8_t *__restrict__ y, int D, int l) {
    float acc = 0.0f;
    for (int d = l; d < D; d += 16) acc = fmaf((float)y[d], q[d], acc);
    return acc;
}

// IP of a code of at most 8 bits, reduced over the half-warp (valid in lane 0).
__device__ __forceinline__ float ip8_half(const float *__restrict__ q, const uint8_t *__restrict__ y, int D, int bits,
                                          int l, unsigned mask) {
    switch (bits) {
    case 1:
        return half_reduce16(chain_bits<1>(q, y, D, l), mask);
    case 2:
        return half_reduce16(chain_bits<2>(q, y, D, l), mask);
    case 3:
        return half_reduce16(chain_bits<3>(q, y, D, l), mask);
    case 4:
        return half_reduce16(chain_bits<4>(q, y, D, l), mask);
    case 5: {  // CodeHelper<5>::compute_ip = 2 * IP4(top 4 bits) + IP1(low bit)
        const float a = half_reduce16(chain_bits<4>(q, y, D, l), mask);
        const float b = half_reduce16(chain_bits<1>(q, y + D / 2, D, l), mask);
        return __fadd_rn(2.0f * a, b);
    }
    case 6:
        return half_reduce16(chain_bits<6>(q, y, D, l), mask);
    case 7:
        return half_reduce16(chain_bits<7>(q, y, D, l), mask);
    case 8:
        return half_reduce16(chain_bits<8>(q, y, D, l), mask);
    default:
        return 0.0f;
    }
}

// get_IP_FUNC(ex_bits)(q, y, D) (code_helper.hpp:599-640) computed by a
// half-warp; result valid in the half's lane 0.
__device__ __forceinline__ float excode_ip_half(const float *__restrict__ q, const uint8_t *__restrict__ y, int D,
                                                int exb, int l, unsigned mask) {
    if (exb == 0) return 0.0f;
    if (exb > 8) {  // CodeHelper<B>::compute_ip, B > 8: IP8(low bytes) + 256 * IP(rest)
        const float lo = ip8_half(q, y, D, 8, l, mask);
        const float hi = ip8_half(q, y + D, D, exb - 8, l, mask);
        return __fadd_rn(lo, 256.0f * hi);
    }
    return ip8_half(q, y, D, exb, l, mask);
}

// ---- the same inner products computed by ONE thread: the 16 SIMD lanes of
// CodeHelper<B>::compute_ip become 16 independent accumulators (lane l takes
// dims l, l+16, ... in increasing order), reduced with the same 16->1 tree.
// Bit-identical to the half-warp form; used where many candidate vectors are
// re-ranked at once (one thread per vector and segment).
__device__ __forceinline__ float tree16(const float *a) {
    float x[8], y[4];
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = __fadd_rn(a[i], a[i + 8]);
#pragma unroll
    for (int i = 0; i < 4; ++i) y[i] = __fadd_rn(x[i], x[i + 4]);
    return __fadd_rn(__fadd_rn(y[0], y[2]), __fadd_rn(y[1], y[3]));
}

template <int B>
__device__ __forceinline__ float ip_thread_bits(const float *__restrict__ q, const uint8_t *__restrict__ y, int D) {
    float acc[16];
#pragma unroll
    for (int l = 0; l < 16; ++l) acc[l] = 0.0f;
    if (B == 1) {
        for (int g = 0; g < D; g += 16) {
            const uint32_t m = (uint32_t)y[g / 8] | ((uint32_t)y[g / 8 + 1] << 8);
#pragma unroll
            for (int l = 0; l < 16; ++l) acc[l] = __fadd_rn(acc[l], ((m >> l) & 1u) ? q[g + l] : 0.0f);
        }
    } else if (B == 2 || B == 3) {
        for (int g = 0; g < D; g += 64) {
            const uint8_t *gp = y + (g / 64) * (B == 2 ? 16 : 24);
            // 16 low-bit bytes; 3-bit groups are 24 bytes, so only 8-byte alignment is guaranteed
            const uint2 w0 = *reinterpret_cast<const uint2 *>(gp), w1 = *reinterpret_cast<const uint2 *>(gp + 8);
            const uint32_t wv[4] = {w0.x, w0.y, w1.x, w1.y};
            uint2 tt = make_uint2(0, 0);
            if (B == 3) tt = *reinterpret_cast<const uint2 *>(gp + 16);
            const uint32_t tv[2] = {tt.x, tt.y};
#pragma unroll
            for (int l = 0; l < 16; ++l) {
                const uint32_t b = (wv[l >> 2] >> (8 * (l & 3))) & 255u;
                const uint32_t t = (tv[(l & 7) >> 2] >> (8 * (l & 3))) & 255u;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    uint32_t v = (b >> (2 * k)) & 3u;
                    if (B == 3) v |= ((t >> (2 * k + (l >> 3))) & 1u) << 2;
                    acc[l] = fmaf((float)v, q[g + 16 * k + l], acc[l]);
                }
            }
        }
    } else if (B == 4) {
        for (int g = 0; g < D; g += 32) {
            const uint4 w = *reinterpret_cast<const uint4 *>(y + (g / 32) * 16);
            const uint32_t wv[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int l = 0; l < 16; ++l) {
                const uint32_t b = (wv[l >> 2] >> (8 * (l & 3))) & 255u;
                acc[l] = fmaf((float)(b & 15u), q[g + l], acc[l]);
                acc[l] = fmaf((float)(b >> 4), q[g + 16 + l], acc[l]);
            }
        }
    } else if (B == 6 || B == 7) {
        for (int g = 0; g < D; g += 64) {
            const uint8_t *gp = y + (g / 64) * (B == 6 ? 48 : 56);
            uint32_t tv[2] = {0, 0};
            if (B == 7) {
                const uint2 tt = *reinterpret_cast<const uint2 *>(gp + 48);
                tv[0] = tt.x;
                tv[1] = tt.y;
            }
#pragma unroll
            for (int l = 0; l < 16; ++l) {
                const uint32_t b0 = gp[l], b1 = gp[16 + l], b2 = gp[32 + l];
                uint32_t v0 = b0 & 63u, v1 = b1 & 63u;
                uint32_t v2 = ((b0 >> 6) << 4) | (b2 & 15u), v3 = ((b1 >> 6) << 4) | (b2 >> 4);
                if (B == 7) {
                    const uint32_t t = (tv[(l & 7) >> 2] >> (8 * (l & 3))) & 255u;
                    const int sh = l >> 3;
                    v0 |= ((t >> (0 + sh)) & 1u) << 6;
                    v1 |= ((t >> (2 + sh)) & 1u) << 6;
                    v2 |= ((t >> (4 + sh)) & 1u) << 6;
                    v3 |= ((t >> (6 + sh)) & 1u) << 6;
                }
                acc[l] = fmaf((float)v0, q[g + l], acc[l]);
                acc[l] = fmaf((float)v1, q[g + 16 + l], acc[l]);
                acc[l] = fmaf((float)v2, q[g + 32 + l], acc[l]);
                acc[l] = fmaf((float)v3, q[g + 48 + l], acc[l]);
            }
        }
    } else {  // 8
        for (int g = 0; g < D; g += 16) {
            const uint4 w = *reinterpret_cast<const uint4 *>(y + g);
            const uint32_t wv[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int l = 0; l < 16; ++l) acc[l] = fmaf((float)((wv[l >> 2] >> (8 * (l & 3))) & 255u), q[g + l], acc[l]);
        }
    }
    return tree16(acc);
}

__device__ __forceinline__ float ip8_thread(const float *__restrict__ q, const uint8_t *__restrict__ y, int D, int bits) {
    switch (bits) {
    case 1:
        return ip_thread_bits<1>(q, y, D);
    case 2:
        return ip_thread_bits<2>(q, y, D);
    case 3:
        return ip_thread_bits<3>(q, y, D);
    case 4:
        return ip_thread_bits<4>(q, y, D);
    case 5:
        return __fadd_rn(2.0f * ip_thread_bits<4>(q, y, D), ip_thread_bits<1>(q, y + D / 2, D));
    case 6:
        return ip_thread_bits<6>(q, y, D);
    case 7:
        return ip_thread_bits<7>(q, y, D);
    case 8:
        return ip_thread_bits<8>(q, y, D);
    default:
        return 0.0f;
    }
}

// get_IP_FUNC(ex_bits)(q, y, D) by one thread.
__device__ __forceinline__ float excode_ip_thread(const float *__restrict__ q, const uint8_t *__restrict__ y, int D,
                                                  int exb) {
    if (exb == 0) return 0.0f;
    if (exb > 8) return __fadd_rn(ip8_thread(q, y, D, 8), 256.0f * ip8_thread(q, y + D, D, exb - 8));
    return ip8_thread(q, y, D, exb);
}

// ---- the same inner products by four lanes: lane j of an aligned group of
// four keeps the SIMD accumulators 4j .. 4j+3 of ip_thread_bits, reading the
// same words, and the group combines them with tree16's pairing (i with i + 8
// and i + 4 across lanes, then (0 + 2) + (1 + 3) in lane 0).  Bit-identical to
// the one-thread form, a quarter of its chain; valid in the group's lane 0.
__device__ __forceinline__ uint32_t pick4(uint32_t a, uint32_t b, uint32_t c, uint32_t d, int j) {
    return j == 0 ? a : j == 1 ? b : j == 2 ? c : d;
}

template <int B>
__device__ __forceinline__ float ip_quad_bits(const float *__restrict__ q, const uint8_t *__restrict__ y, int D, int j) {
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const int l0 = 4 * j;
    if (B == 1) {
        for (int g = 0; g < D; g += 16) {
            const uint32_t m = (uint32_t)y[g / 8] | ((uint32_t)y[g / 8 + 1] << 8);
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
                const int l = l0 + jj;
                acc[jj] = __fadd_rn(acc[jj], ((m >> l) & 1u) ? q[g + l] : 0.0f);
            }
        }
    } else if (B == 2 || B == 3) {
        for (int g = 0; g < D; g += 64) {
            const uint8_t *gp = y + (g / 64) * (B == 2 ? 16 : 24);
            const uint2 w0 = *reinterpret_cast<const uint2 *>(gp), w1 = *reinterpret_cast<const uint2 *>(gp + 8);
            const uint32_t w = pick4(w0.x, w0.y, w1.x, w1.y, j);
            uint32_t tw = 0;
            if (B == 3) {
                const uint2 tt = *reinterpret_cast<const uint2 *>(gp + 16);
                tw = (j & 1) ? tt.y : tt.x;  // word (l & 7) >> 2 of the top bits
            }
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
                const int l = l0 + jj;
                const uint32_t b = (w >> (8 * jj)) & 255u;
                const uint32_t t = (tw >> (8 * jj)) & 255u;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    uint32_t v = (b >> (2 * k)) & 3u;
                    if (B == 3) v |= ((t >> (2 * k + (l >> 3))) & 1u) << 2;
                    acc[jj] = fmaf((float)v, q[g + 16 * k + l], acc[jj]);
                }
            }
        }
    } else if (B == 4) {
        for (int g = 0; g < D; g += 32) {
            const uint4 w4 = *reinterpret_cast<const uint4 *>(y + (g / 32) * 16);
            const uint32_t w = pick4(w4.x, w4.y, w4.z, w4.w, j);
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
                const int l = l0 + jj;
                const uint32_t b = (w >> (8 * jj)) & 255u;
                acc[jj] = fmaf((float)(b & 15u), q[g + l], acc[jj]);
                acc[jj] = fmaf((float)(b >> 4), q[g + 16 + l], acc[jj]);
            }
        }
    } else if (B == 6 || B == 7) {
        for (int g = 0; g < D; g += 64) {
            const uint8_t *gp = y + (g / 64) * (B == 6 ? 48 : 56);
            uint32_t tw = 0;
            if (B == 7) {
                const uint2 tt = *reinterpret_cast<const uint2 *>(gp + 48);
                tw = (j & 1) ? tt.y : tt.x;
            }
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
                const int l = l0 + jj;
                const uint32_t b0 = gp[l], b1 = gp[16 + l], b2 = gp[32 + l];
                uint32_t v0 = b0 & 63u, v1 = b1 & 63u;
                uint32_t v2 = ((b0 >> 6) << 4) | (b2 & 15u), v3 = ((b1 >> 6) << 4) | (b2 >> 4);
                if (B == 7) {
                    const uint32_t t = (tw >> (8 * jj)) & 255u;
                    const int sh = l >> 3;
                    v0 |= ((t >> (0 + sh)) & 1u) << 6;
                    v1 |= ((t >> (2 + sh)) & 1u) << 6;
                    v2 |= ((t >> (4 + sh)) & 1u) << 6;
                    v3 |= ((t >> (6 + sh)) & 1u) << 6;
                }
                acc[jj] = fmaf((float)v0, q[g + l], acc[jj]);
                acc[jj] = fmaf((float)v1, q[g + 16 + l], acc[jj]);
                acc[jj] = fmaf((float)v2, q[g + 32 + l], acc[jj]);
                acc[jj] = fmaf((float)v3, q[g + 48 + l], acc[jj]);
            }
        }
    } else {  // 8
        for (int g = 0; g < D; g += 16) {
            const uint4 w4 = *reinterpret_cast<const uint4 *>(y + g);
            const uint32_t w = pick4(w4.x, w4.y, w4.z, w4.w, j);
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) acc[jj] = fmaf((float)((w >> (8 * jj)) & 255u), q[g + l0 + jj], acc[jj]);
        }
    }
    // tree16: x[i] = a[i] + a[i + 8] (lanes 0, 1 with lanes 2, 3), y[i] = x[i] + x[i + 4]
    // (lane 0 with lane 1), then (y0 + y2) + (y1 + y3)
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) acc[jj] = __fadd_rn(acc[jj], __shfl_down_sync(kFull, acc[jj], 2, 4));
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) acc[jj] = __fadd_rn(acc[jj], __shfl_down_sync(kFull, acc[jj], 1, 4));
    return __fadd_rn(__fadd_rn(acc[0], acc[2]), __fadd_rn(acc[1], acc[3]));
}

__device__ __forceinline__ float ip8_quad(const float *__restrict__ q, const uint8_t *__restrict__ y, int D, int bits,
                                          int j) {
    switch (bits) {
    case 1:
        return ip_quad_bits<1>(q, y, D, j);
    case 2:
        return ip_quad_bits<2>(q, y, D, j);
    case 3:
        return ip_quad_bits<3>(q, y, D, j);
    case 4:
        return ip_quad_bits<4>(q, y, D, j);
    case 5:  // CodeHelper<5>::compute_ip = 2 * IP4(top 4 bits) + IP1(low bit)
        return __fadd_rn(2.0f * ip_quad_bits<4>(q, y, D, j), ip_quad_bits<1>(q, y + D / 2, D, j));
    case 6:
        return ip_quad_bits<6>(q, y, D, j);
    case 7:
        return ip_quad_bits<7>(q, y, D, j);
    case 8:
        return ip_quad_bits<8>(q, y, D, j);
    default:
        return 0.0f;
    }
}

// get_IP_FUNC(ex_bits)(q, y, D) by an aligned group of four lanes (j = lane & 3;
// every lane of the warp takes part); valid in the group's lane 0.
__device__ __forceinline__ float excode_ip_quad(const float *__restrict__ q, const uint8_t *__restrict__ y, int D,
                                                int exb, int j) {
    if (exb == 0) return 0.0f;
    if (exb > 8) return __fadd_rn(ip8_quad(q, y, D, 8, j), 256.0f * ip8_quad(q, y + D, D, exb - 8, j));
    return ip8_quad(q, y, D, exb, j);
}

// CaqCluEstimator::compAccurateDist + Lut::getExtIP, L2 (caq_estimator.hpp:190-217, lut.hpp:121-126)
__device__ __forceinline__ float accurate_dist(float onorm, float ipx, float ex_ip, float rescale, int bits, float sum_q,
                                               float q_l2sqr) {
    const float o2 = __fmul_rn(onorm, onorm);
    if (bits == 0) return __fadd_rn(o2, q_l2sqr);
    const float dl = (float)(2.0 / (double)(1 << bits));
    const double e = __dadd_rn(__dadd_rn((double)ipx, __dmul_rn((double)ex_ip, (double)dl)),
                               __dmul_rn(__dadd_rn(-1.0, (double)(dl / 2)), (double)sum_q));
    const float ipoq = __fmul_rn(rescale, (float)e);
    return __fsub_rn(__fadd_rn(o2, q_l2sqr), __fmul_rn(2.0f, ipoq));
}

}  // namespace saqg
