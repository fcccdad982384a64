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
// Value of dimension d in the reference's compacted ex-code layouts
// (utils/code_helper.hpp CodeHelper<B>::compacted_code8, B <= 8).
__device__ __forceinline__ uint32_t excode_get8(const uint8_t *__restrict__ y, int d, int bits) {
    switch (bits) {
    case 1:
        return (y[d >> 3] >> (d & 7)) & 1u;
    case 2: {
        const int g = d >> 6, k = d & 63;
        return (y[g * 16 + (k & 15)] >> (2 * (k >> 4))) & 3u;
    }
    case 3: {
        const int g = d >> 6, k = d & 63;
        const uint8_t *b = y + g * 24;
        return ((b[k & 15] >> (2 * (k >> 4))) & 3u) | (((b[16 + (k & 7)] >> (k >> 3)) & 1u) << 2);
    }
    case 4: {
        const int g = d >> 5, k = d & 31;
        const uint8_t byte = y[g * 16 + (k & 15)];
        return k < 16 ? (byte & 15u) : (uint32_t)(byte >> 4);
    }
    case 6:
    case 7: {
        const int g = d >> 6, k = d & 63, r = k & 15;
        const uint8_t *b = y + g * (bits == 6 ? 48 : 56);
        uint32_t v;
        if (k < 16) v = b[r] & 63u;
        else if (k < 32) v = b[16 + r] & 63u;
        else if (k < 48) v = ((uint32_t)(b[r] >> 6) << 4) | (b[32 + r] & 15u);
        else v = ((uint32_t)(b[16 + r] >> 6) << 4) | (uint32_t)(b[32 + r] >> 4);
        if (bits == 7) v |= ((b[48 + (k & 7)] >> (k >> 3)) & 1u) << 6;
        return v;
    }
    case 8:
        return y[d];
    default:
        return 0;
    }
}

// One 16-lane chain of CodeHelper<bits>::compute_ip for bits in 1..8 except 5,
// run by half-warp lane l (dims l, l+16, ...).  Returns this lane's accumulator.
__device__ __forceinline__ float excode_lane_chain(const float *__restrict__ q, const uint8_t *__restrict__ y, int D,
                                                   int bits, int l) {
    float acc = 0.0f;
    if (bits == 1) {
        for (int d = l; d < D; d += 16) acc = __fadd_rn(acc, excode_get8(y, d, 1) ? q[d] : 0.0f);
    } else {
        for (int d = l; d < D; d += 16) acc = fmaf((float)excode_get8(y, d, bits), q[d], acc);
    }
    return acc;
}

// get_IP_FUNC(ex_bits)(q, y, D) (code_helper.hpp:599-640) computed by a
// half-warp; result valid in the half's lane 0.
__device__ __forceinline__ float excode_ip_half(const float *__restrict__ q, const uint8_t *__restrict__ y, int D,
                                                int exb, int l, unsigned mask) {
    if (exb == 0) return 0.0f;
    if (exb > 8) {  // CodeHelper<B>::compute_ip, B > 8: IP8(low bytes) + 256 * IP(rest)
        float lo = half_reduce16(excode_lane_chain(q, y, D, 8, l), mask);
        float hi;
        const int hb = exb - 8;
        if (hb == 5) {
            float a = half_reduce16(excode_lane_chain(q, y + D, D, 4, l), mask);
            float b = half_reduce16(excode_lane_chain(q, y + D + D / 2, D, 1, l), mask);
            hi = __fadd_rn(2.0f * a, b);
        } else {
            hi = half_reduce16(excode_lane_chain(q, y + D, D, hb, l), mask);
        }
        return __fadd_rn(lo, 256.0f * hi);
    }
    if (exb == 5) {  // CodeHelper<5>::compute_ip = 2 * IP4(top 4 bits) + IP1(low bit)
        float a = half_reduce16(excode_lane_chain(q, y, D, 4, l), mask);
        float b = half_reduce16(excode_lane_chain(q, y + D / 2, D, 1, l), mask);
        return __fadd_rn(2.0f * a, b);
    }
    return half_reduce16(excode_lane_chain(q, y, D, exb, l), mask);
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
