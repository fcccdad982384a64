// CPU ORACLE -- test infrastructure only, never part of the product.
//
// A scalar C++ restatement of SAQ's search and encode hot path (howarlii/SAQ,
// saqlib/) used (1) as the parity checker for the CUDA path and (2) as the
// timed CPU baseline ("port").  It runs on any host (x86 or Arm) and is pinned
// against golden vectors produced by the reference itself (tests/golden/).
//
// Floating-point order.  The reference is compiled with -O3 -march=native
// -ffp-contract=off on an AVX-512 host, so its float results depend on the
// fixed SIMD evaluation order of Eigen 3.4 and of GCC's _mm512 reductions.
// Those orders are restated here lane by lane:
//   * eigen_sum*   : Eigen redux_impl<LinearVectorizedTraversal> (Redux.h:227-283):
//                    two 16-lane accumulators over even/odd packets, merged,
//                    an optional odd packet, predux (16->8->4->2->1), scalar tail.
//   * reduce16     : GCC _mm512_reduce_add_ps / Eigen predux<Packet16f>:
//                    lane i + lane i+8, then +4, +2, +1.
//   * gemv_rowvec  : Eigen general_matrix_vector_product<ColMajor> (GeneralMatrixVector.h:108-300)
//                    reached by RowVector * RowMajor matrix: for each output, FMA
//                    chains over blocks of 16 input rows (whole input if D < 128),
//                    block partial sums added in order.
//   * excode ip    : CodeHelper<B>::compute_ip (utils/code_helper.hpp): 16 lanes,
//                    lane l accumulates dims d = l (mod 16) in increasing d with FMA
//                    (plain adds for B=1), then reduce16.
// Build with -ffp-contract=off so that no a*b+c is fused behind our back; FMAs
// are explicit std::fma calls.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

namespace {

constexpr int kFS = 32;  // vectors per FastScan block (defines.hpp KFastScanSize)

// ------------------------------------------------------------------ reductions
inline float reduce16(const float *p) {
    float x[8], y[4];
    for (int i = 0; i < 8; ++i) x[i] = p[i] + p[i + 8];
    for (int i = 0; i < 4; ++i) y[i] = x[i] + x[i + 4];
    float z0 = y[0] + y[2], z1 = y[1] + y[3];
    return z0 + z1;
}

// Eigen redux over n elements produced by f(i) (elements are computed with
// their own rounding before being summed).
template <class F>
inline float eigen_redux_sum(long n, F f) {
    const long P = 16;
    long aligned = n / P * P, aligned2 = n / (2 * P) * (2 * P);
    if (aligned == 0) {
        float r = f(0);
        for (long i = 1; i < n; ++i) r = r + f(i);
        return r;
    }
    float r0[16], r1[16];
    for (int l = 0; l < 16; ++l) r0[l] = f(l);
    if (aligned > P) {
        for (int l = 0; l < 16; ++l) r1[l] = f(P + l);
        for (long idx = 2 * P; idx < aligned2; idx += 2 * P)
            for (int l = 0; l < 16; ++l) {
                r0[l] = r0[l] + f(idx + l);
                r1[l] = r1[l] + f(idx + P + l);
            }
        for (int l = 0; l < 16; ++l) r0[l] = r0[l] + r1[l];
        if (aligned > aligned2)
            for (int l = 0; l < 16; ++l) r0[l] = r0[l] + f(aligned2 + l);
    }
    float r = reduce16(r0);
    for (long i = aligned; i < n; ++i) r = r + f(i);
    return r;
}

inline float eigen_sum(const float *x, long n) { return eigen_redux_sum(n, [&](long i) { return x[i]; }); }
inline float eigen_sqnorm(const float *x, long n) {
    return eigen_redux_sum(n, [&](long i) { return x[i] * x[i]; });
}
inline float eigen_dot(const float *a, const float *b, long n) {
    return eigen_redux_sum(n, [&](long i) { return a[i] * b[i]; });
}
inline float eigen_sqdist(const float *a, const float *b, long n) {
    return eigen_redux_sum(n, [&](long i) {
        float d = a[i] - b[i];
        return d * d;
    });
}
// (var .* q.^2).sum() as in saq_estimator.hpp:42-44
inline float eigen_var_q2(const float *var, const float *q, long n) {
    return eigen_redux_sum(n, [&](long i) { return var[i] * (q[i] * q[i]); });
}

// out = Q * P for m row vectors Q (m x D) and P (D x D, row-major).  Per
// output (r, i) the arithmetic is
//   res = 0; for each block b of bc inputs: c = 0; c = fma(P[j][i], Q[r][j], c)
//   for j ascending in b; res = fma(c, 1, res)
// i.e. Eigen's GEMV order for each row.  The loops run input-row-major (all
// outputs of all m rows advance together over one row of P, which is read once
// per m vectors); every output still sees exactly the sequence above.  `out`
// must not alias `Q`.
void gemv_rows(const float *Q, long m, const float *P, long D, float *out) {
    const long bc = D < 128 ? D : 16;
    constexpr long kW = 64;  // outputs held in registers across one block's inputs
    for (long i = 0; i < m * D; ++i) out[i] = 0.0f;
    for (long j2 = 0; j2 < D; j2 += bc) {
        const long je = std::min(j2 + bc, D);
        for (long r = 0; r < m; ++r) {
            const float *q = Q + r * D;
            float *o = out + r * D;
            long i0 = 0;
            for (; i0 + kW <= D; i0 += kW) {
                float c[kW];
                for (long t = 0; t < kW; ++t) c[t] = 0.0f;
                for (long j = j2; j < je; ++j) {
                    const float qj = q[j];
                    const float *row = P + j * D + i0;
                    for (long t = 0; t < kW; ++t) c[t] = std::fma(row[t], qj, c[t]);
                }
                for (long t = 0; t < kW; ++t) o[i0 + t] = std::fma(c[t], 1.0f, o[i0 + t]);
            }
            for (long i = i0; i < D; ++i) {
                float c = 0.0f;
                for (long j = j2; j < je; ++j) c = std::fma(P[j * D + i], q[j], c);
                o[i] = std::fma(c, 1.0f, o[i]);
            }
        }
    }
}

// out = q (1 x D) * P (D x D, row-major), Eigen's GEMV order (gemv_rows with m = 1).
void gemv_rowvec(const float *q, const float *P, long D, float *out) { gemv_rows(q, 1, P, D, out); }

// x86 minps semantics: (a < b) ? a : b
inline float minps(float a, float b) { return a < b ? a : b; }
inline float maxps(float a, float b) { return a > b ? a : b; }

// _mm512_reduce_min_ps(_mm512_min_ps(d0, d1)) (saq_searcher.hpp:105,128)
float reduce_min32(const float *d) {
    float v[16];
    for (int i = 0; i < 16; ++i) v[i] = minps(d[i], d[16 + i]);
    float t3[8], t6[4];
    for (int i = 0; i < 8; ++i) t3[i] = minps(v[8 + i], v[i]);
    for (int i = 0; i < 4; ++i) t6[i] = minps(t3[4 + i], t3[i]);
    float t8_0 = minps(t6[0], t6[2]), t8_1 = minps(t6[1], t6[3]);
    return minps(t8_0, t8_1);
}

// ---------------------------------------------------------- ex-code layouts
// Layouts written by CodeHelper<B>::compacted_code8/16 (code_helper.hpp:17-568).
// unpack: packed bytes -> per-dimension value of `bits` bits.
void unpack_bits8(const uint8_t *y, long D, int bits, uint16_t *out) {
    switch (bits) {
    case 0:
        for (long d = 0; d < D; ++d) out[d] = 0;
        return;
    case 1:
        for (long d = 0; d < D; ++d) out[d] = (y[d / 8] >> (d % 8)) & 1;
        return;
    case 2:
    case 3:
        for (long g = 0; g < D / 64; ++g) {
            const uint8_t *b = y + g * (bits == 2 ? 16 : 24);
            for (int k = 0; k < 64; ++k) {
                uint16_t v = (b[k % 16] >> (2 * (k / 16))) & 3;
                if (bits == 3) v |= ((b[16 + (k % 8)] >> (k / 8)) & 1) << 2;
                out[g * 64 + k] = v;
            }
        }
        return;
    case 4:
        for (long g = 0; g < D / 32; ++g) {
            const uint8_t *b = y + g * 16;
            for (int k = 0; k < 32; ++k) out[g * 32 + k] = k < 16 ? (b[k] & 15) : (b[k - 16] >> 4);
        }
        return;
    case 5: {
        std::vector<uint16_t> hi(D), lo(D);
        unpack_bits8(y, D, 4, hi.data());
        unpack_bits8(y + D * 4 / 8, D, 1, lo.data());
        for (long d = 0; d < D; ++d) out[d] = (hi[d] << 1) | lo[d];
        return;
    }
    case 6:
    case 7:
        for (long g = 0; g < D / 64; ++g) {
            const uint8_t *b = y + g * (bits == 6 ? 48 : 56);
            for (int k = 0; k < 64; ++k) {
                int r = k % 16;
                uint16_t v;
                if (k < 16) v = b[r] & 63;
                else if (k < 32) v = b[16 + r] & 63;
                else if (k < 48) v = ((b[r] >> 6) << 4) | (b[32 + r] & 15);
                else v = ((b[16 + r] >> 6) << 4) | (b[32 + r] >> 4);
                if (bits == 7) v |= ((b[48 + (k % 8)] >> (k / 8)) & 1) << 6;
                out[g * 64 + k] = v;
            }
        }
        return;
    case 8:
        for (long d = 0; d < D; ++d) out[d] = y[d];
        return;
    default:
        std::abort();
    }
}

void pack_bits8(const uint16_t *v, long D, int bits, uint8_t *y) {
    switch (bits) {
    case 0:
        return;
    case 1:
        for (long i = 0; i < D / 8; ++i) {
            uint8_t b = 0;
            for (int j = 0; j < 8; ++j) b |= (v[i * 8 + j] & 1) << j;
            y[i] = b;
        }
        return;
    case 2:
    case 3:
        for (long g = 0; g < D / 64; ++g) {
            uint8_t *b = y + g * (bits == 2 ? 16 : 24);
            const uint16_t *c = v + g * 64;
            for (int r = 0; r < 16; ++r)
                b[r] = (c[r] & 3) | ((c[16 + r] & 3) << 2) | ((c[32 + r] & 3) << 4) | ((c[48 + r] & 3) << 6);
            if (bits == 3)
                for (int k = 0; k < 8; ++k) {
                    uint8_t t = 0;
                    for (int m = 0; m < 8; ++m) t |= ((c[8 * m + k] >> 2) & 1) << m;
                    b[16 + k] = t;
                }
        }
        return;
    case 4:
        for (long g = 0; g < D / 32; ++g)
            for (int r = 0; r < 16; ++r) y[g * 16 + r] = (v[g * 32 + r] & 15) | ((v[g * 32 + 16 + r] & 15) << 4);
        return;
    case 5: {
        std::vector<uint16_t> hi(D);
        for (long d = 0; d < D; ++d) hi[d] = v[d] >> 1;
        pack_bits8(hi.data(), D, 4, y);
        pack_bits8(v, D, 1, y + D * 4 / 8);
        return;
    }
    case 6:
    case 7:
        for (long g = 0; g < D / 64; ++g) {
            uint8_t *b = y + g * (bits == 6 ? 48 : 56);
            const uint16_t *c = v + g * 64;
            for (int r = 0; r < 16; ++r) {
                b[r] = (c[r] & 63) | (((c[32 + r] >> 4) & 3) << 6);
                b[16 + r] = (c[16 + r] & 63) | (((c[48 + r] >> 4) & 3) << 6);
                b[32 + r] = (c[32 + r] & 15) | ((c[48 + r] & 15) << 4);
            }
            if (bits == 7)
                for (int k = 0; k < 8; ++k) {
                    uint8_t t = 0;
                    for (int m = 0; m < 8; ++m) t |= ((c[8 * m + k] >> 6) & 1) << m;
                    b[48 + k] = t;
                }
        }
        return;
    case 8:
        for (long d = 0; d < D; ++d) y[d] = (uint8_t)v[d];
        return;
    default:
        std::abort();
    }
}

// compacted_code16: >8 bits = low bytes (D) followed by the 8-bit layout of the rest.
void pack_excode(const uint16_t *v, long D, int bits, uint8_t *y) {
    if (bits > 8) {
        std::vector<uint16_t> hi(D);
        for (long d = 0; d < D; ++d) {
            y[d] = v[d] & 0xFF;
            hi[d] = v[d] >> 8;
        }
        pack_bits8(hi.data(), D, bits - 8, y + D);
    } else {
        pack_bits8(v, D, bits, y);
    }
}

void unpack_excode(const uint8_t *y, long D, int bits, uint16_t *v) {
    if (bits > 8) {
        std::vector<uint16_t> hi(D);
        unpack_bits8(y + D, D, bits - 8, hi.data());
        for (long d = 0; d < D; ++d) v[d] = y[d] | (hi[d] << 8);
    } else {
        unpack_bits8(y, D, bits, v);
    }
}

// 16-lane FMA chains + reduce16 over a code of up to 8 bits (CodeHelper<2..8>)
float lanes_fma_ip(const float *q, const uint16_t *c, long D) {
    float lane[16] = {0};
    for (long d = 0; d < D; ++d) lane[d % 16] = std::fma((float)c[d], q[d], lane[d % 16]);
    return reduce16(lane);
}
// CodeHelper<1>::compute_ip: masked adds
float lanes_mask_ip(const float *q, const uint16_t *c, long D) {
    float lane[16] = {0};
    for (long d = 0; d < D; ++d) lane[d % 16] = lane[d % 16] + ((c[d] & 1) ? q[d] : 0.0f);
    return reduce16(lane);
}

float ip8(const float *q, const uint8_t *y, long D, int bits) {
    if (bits == 0) return 0.0f;
    std::vector<uint16_t> c(D);
    if (bits == 5) {
        // CodeHelper<5>::compute_ip = 2*IP4(top 4 bits) + IP1(low bit)  (code_helper.hpp:371-374)
        unpack_bits8(y, D, 4, c.data());
        float a = lanes_fma_ip(q, c.data(), D);
        unpack_bits8(y + D * 4 / 8, D, 1, c.data());
        float b = lanes_mask_ip(q, c.data(), D);
        return 2 * a + b;
    }
    unpack_bits8(y, D, bits, c.data());
    return bits == 1 ? lanes_mask_ip(q, c.data(), D) : lanes_fma_ip(q, c.data(), D);
}

// get_IP_FUNC(bits) (code_helper.hpp:599-640); >8 bits: IP8(low) + 256*IP(rest)
float excode_ip(const float *q, const uint8_t *y, long D, int bits) {
    if (bits > 8) return ip8(q, y, D, 8) + 256 * ip8(q, y + D, D, bits - 8);
    return ip8(q, y, D, bits);
}

// ------------------------------------------------------------------ FastScan
// kPerm0 / pack_codes (fastscan.hpp:41-112): per 8-dim column, 16 bytes for the
// high-nibble codebook then 16 for the low one; byte j holds vector kPerm0[j]
// in its low nibble and vector kPerm0[j]+16 in its high nibble.
const int kPerm0[16] = {0, 8, 1, 9, 2, 10, 3, 11, 4, 12, 5, 13, 6, 14, 7, 15};
const int kPos[16] = {3, 3, 2, 3, 1, 3, 2, 3, 0, 3, 2, 3, 1, 3, 2, 3};

void pack_block(const uint8_t *sc /*32 x D/8*/, long D, uint8_t *blk /*4D*/) {
    long cols = D / 8;
    for (long i = 0; i < cols; ++i) {
        uint8_t c0[32], c1[32];
        for (int j = 0; j < 32; ++j) {
            uint8_t b = sc[j * cols + i];
            c0[j] = b >> 4;
            c1[j] = b & 15;
        }
        for (int j = 0; j < 16; ++j) {
            blk[i * 32 + j] = c0[kPerm0[j]] | (c0[kPerm0[j] + 16] << 4);
            blk[i * 32 + 16 + j] = c1[kPerm0[j]] | (c1[kPerm0[j] + 16] << 4);
        }
    }
}

// nibble (4-bit code of codebook cb) of vector v in a packed block
inline int block_nibble(const uint8_t *blk, long cb, int v) {
    int r = v & 15;
    int j = r < 8 ? 2 * r : 2 * (r - 8) + 1;
    uint8_t b = blk[(cb / 2) * 32 + (cb & 1) * 16 + j];
    return v < 16 ? (b & 15) : (b >> 4);
}

// ------------------------------------------------------------------ planner
struct Plan {
    std::vector<std::pair<long, long>> segs;
};

Plan plan_dp(const float *var, long Dp, float avg_bits) {
    const size_t nbf = 2 * sizeof(float) * 8;  // 64 bits of short factors per segment
    const size_t tot_bits = (size_t)(avg_bits * (float)Dp + (float)nbf);
    const size_t max_ns = avg_bits < 2 ? Dp / 64 : Dp / 64 / 2;
    const size_t i_end = Dp / 64;
    const double lim = std::numeric_limits<double>::max();
    const size_t W = tot_bits + 1, H = i_end + 1;
    std::vector<double> fv((max_ns + 1) * H * W, lim);
    std::vector<size_t> fs((max_ns + 1) * H * W, 0);
    auto at = [&](size_t ns, size_t i, size_t b) { return (ns * H + i) * W + b; };
    size_t ans_ns = 0, ans_i = i_end, ans_b = tot_bits;
    fv[at(0, 0, 0)] = 0;
    std::vector<float> blk_sum(i_end);
    for (size_t i = 0; i < i_end; ++i) blk_sum[i] = eigen_sum(var + i * 64, 64);
    for (size_t ns = 0; ns <= max_ns; ns++)
        for (size_t i = 0; i <= i_end; i++)
            for (size_t ub = 0; ub <= tot_bits; ++ub) {
                double cur = fv[at(ns, i, ub)];
                if (!(cur < lim)) continue;
                if (i == i_end) {
                    if (cur * (1.01) < fv[at(ans_ns, ans_i, ans_b)]) {
                        ans_ns = ns;
                        ans_i = i;
                        ans_b = ub;
                    }
                    continue;
                }
                if (ns == max_ns) continue;
                double var_sum = 0;
                for (size_t j = 1; (i + j) * 64 <= (size_t)Dp; j++) {
                    var_sum += blk_sum[i + j - 1];
                    for (size_t b = 1; b <= 13; ++b) {
                        size_t Bn = ub + b * j * 64 + nbf;
                        if (Bn > tot_bits) break;
                        double v = var_sum / (1 << b);
                        size_t t = at(ns + 1, i + j, Bn);
                        if (fv[t] > cur + v) {
                            fv[t] = cur + v;
                            fs[t] = (i << 4) + b;
                        }
                    }
                }
                size_t t = at(ns + 1, i_end, ub);
                if (cur + var_sum < fv[t]) {
                    fv[t] = cur + var_sum;
                    fs[t] = (i << 4) + 0;
                }
            }
    Plan p;
    size_t ns = ans_ns, i = ans_i, B = ans_b;
    while (i > 0) {
        size_t s = fs[at(ns, i, B)];
        size_t pi = s >> 4, bits = s & 0xf, len = (i - pi) * 64;
        p.segs.emplace_back(len, bits);
        ns--;
        i = pi;
        if (bits) B -= bits * len + nbf;
    }
    std::reverse(p.segs.begin(), p.segs.end());
    return p;
}

Plan plan_equal(long Dp, float avg_bits, int nseg) {
    Plan p;
    size_t b = (size_t)avg_bits;
    long d = 0;
    for (int i = 0; i < nseg && d < Dp; i++) {
        long t = ((Dp - d) / (nseg - i) + 63) / 64 * 64;
        p.segs.emplace_back(t, b);
        d += t;
    }
    return p;
}

// ------------------------------------------------------------------ encoder
struct CaqOut {
    std::vector<int> code;
    float o_l2norm, ip_cent_oa, rescale, error;
};

// CAQEncoder::encode + code_adjustment + encode_and_fac (caq_encoder.hpp:57-247)
void caq_encode(const float *o, long D, int bits, const float *cent_unrot, int rdlmt, float eps, CaqOut &out) {
    out.code.assign(D, 0);
    double v_mx = 0, v_mi = 0, delta = 0, ip = 0, oa2 = 0;
    if (bits > 0) {
        const int cmax = (1 << bits) - 1;
        float mx = o[0], mn = o[0];
        for (long j = 1; j < D; ++j) {
            mx = std::max(mx, o[j]);
            mn = std::min(mn, o[j]);
        }
        v_mx = std::max(mx, -mn);
        v_mi = -v_mx;
        delta = (v_mx - v_mi) / (cmax + 1);
        double vec_sum = eigen_sum(o, D);
        std::vector<float> cf(D, 0.0f);
        if (delta != 0) {
            const float vmi_f = (float)v_mi, d_f = (float)delta;
            for (long j = 0; j < D; ++j) cf[j] = std::min(std::floor((o[j] - vmi_f) / d_f), (float)cmax);
        }
        double ip_o_code = 0;
        uint64_t code_l2 = 0;
        for (long j = 0; j < D; ++j) {
            ip_o_code += (double)(cf[j] * o[j]);
            int c = (int)cf[j];
            out.code[j] = c;
            code_l2 += (uint64_t)(c * c);
        }
        uint32_t code_sum = 0;
        for (long j = 0; j < D; ++j) code_sum += (uint32_t)out.code[j];
        ip = ip_o_code * delta + (v_mi + 0.5 * delta) * vec_sum;
        oa2 = delta * delta * (double)code_l2 + (delta * delta + 2 * delta * v_mi) * (double)code_sum;
        oa2 += (0.25 * delta * delta + delta * v_mi + v_mi * v_mi) * (double)D;
        if (rdlmt && oa2 != 0) {
            const double re_eps = (double)eps * oa2;
            for (int adj = 1, round = 1; adj; round++) {
                adj = 0;
                for (long j = 0; j < D; ++j) {
                    int cur = 0;
                    const float ov = o[j];
                    double oa = (out.code[j] + 0.5) * delta + v_mi;
                    int c = out.code[j];
                    const double tmp = oa2 - oa * oa;
                    const double ipd = delta * ov;
                    while (c < cmax) {
                        double nq = oa + delta, nl = tmp + nq * nq, ni = ip + ipd;
                        if ((ip * ip + re_eps) * nl >= ni * ni * oa2) break;
                        c++;
                        ip = ni;
                        oa = nq;
                        oa2 = nl;
                        cur++;
                    }
                    while (c > 0) {
                        double nq = oa - delta, nl = tmp + nq * nq, ni = ip - ipd;
                        if ((ip * ip + re_eps) * nl >= ni * ni * oa2) break;
                        c--;
                        ip = ni;
                        oa = nq;
                        oa2 = nl;
                        cur++;
                    }
                    if (out.code[j] != c) {
                        out.code[j] = c;
                        adj += cur;
                    }
                }
                if (rdlmt && round >= rdlmt) break;
                double ci = 0, co = 0;
                for (long j = 0; j < D; ++j) {
                    double q = (out.code[j] + 0.5) * delta + v_mi;
                    ci += q * o[j];
                    co += q * q;
                }
                oa2 = co;
                ip = ci;
            }
        }
    }
    const double o_l2sqr = eigen_sqnorm(o, D);
    const double o_l2norm = std::sqrt(o_l2sqr);
    double rescale = ip ? o_l2sqr / ip : 0;
    double err = o_l2sqr * (double)1.9f * std::sqrt((((o_l2sqr * oa2) / (ip * ip)) - 1) / (double)(D - 1));
    if (v_mx) {
        const double s = 1.0 / v_mx;
        delta *= s;
        ip *= s;
        oa2 *= s * s;
        rescale *= v_mx;
        v_mi *= s;
        v_mx *= s;
    }
    out.o_l2norm = (float)o_l2norm;
    out.rescale = (float)rescale;
    out.error = (float)err;
    out.ip_cent_oa = 0;
    if (bits > 1 && cent_unrot) {
        std::vector<float> oav(D);
        const float df = (float)delta, vf = (float)v_mi;
        for (long j = 0; j < D; ++j) oav[j] = (float)out.code[j] * df + vf;
        out.ip_cent_oa = eigen_dot(cent_unrot, oav.data(), D);
    }
}

// ------------------------------------------------------------------ index
struct Seg {
    long dim, bits;
    std::vector<float> P;  // empty -> no rotation
};
struct Clu {
    long n, nb;
    std::vector<float> sfac;   // multi-seg short factors
    std::vector<uint8_t> scode;
    std::vector<uint8_t> lcode;
    std::vector<float> lfac;   // n x S x 2
    std::vector<uint32_t> ids;
    std::vector<std::vector<float>> cent;  // per segment rotated centroid
};
struct Index {
    long N = 0, D = 0, K = 0;
    std::vector<float> centroids;
    uint8_t qcfg[32] = {0};
    std::vector<float> var;
    std::vector<Seg> segs;
    std::vector<Clu> clus;
    bool compact = true;
    // derived
    std::vector<long> sc_bytes, long_pv, long_off;  // per segment
    long block_bytes = 0, long_stride = 0;
    std::vector<long> sc_off;  // offset of segment codes inside a (multi-seg) code block
    void derive() {
        long S = (long)segs.size();
        compact = S == 1 || qcfg[9] != 0;
        sc_bytes.assign(S, 0);
        long_pv.assign(S, 0);
        long_off.assign(S, 0);
        sc_off.assign(S, 0);
        block_bytes = 0;
        long_stride = 0;
        for (long s = 0; s < S; ++s) {
            sc_bytes[s] = segs[s].bits ? segs[s].dim * kFS / 8 : 0;
            long_pv[s] = segs[s].bits ? segs[s].dim * (segs[s].bits - 1) / 8 : 0;
        }
        if (S == 1) {
            block_bytes = 64 * 4 + sc_bytes[0];
            long_stride = long_pv[0];
        } else {
            for (long s = 0; s < S; ++s) {
                sc_off[s] = block_bytes;
                block_bytes += sc_bytes[s];
                long_off[s] = long_stride;
                long_stride += compact ? long_pv[s] : (long_pv[s] + 15) / 16 * 16;
            }
        }
    }
    // accessors mirroring CAQClusterData (cluster_data.hpp:106-141)
    const float *onorm(const Clu &c, long s, long b) const {
        if (segs.size() == 1) return reinterpret_cast<const float *>(c.scode.data() + b * block_bytes);
        return c.sfac.data() + b * 64 * segs.size() + s * 64;
    }
    const uint8_t *codes(const Clu &c, long s, long b) const {
        if (segs.size() == 1) return c.scode.data() + b * block_bytes + 256;
        return c.scode.data() + b * block_bytes + sc_off[s];
    }
    const uint8_t *lcode(const Clu &c, long s, long v) const {
        if (segs.size() == 1) return c.lcode.data() + v * long_pv[0];
        if (compact) {
            // segment-major arrays, each padded to 16 bytes (cluster_data.hpp:281-284)
            long off = 0;
            for (long t = 0; t < s; ++t) off += (long_pv[t] * c.n + 15) / 16 * 16;
            return c.lcode.data() + off + v * long_pv[s];
        }
        return c.lcode.data() + v * long_stride + long_off[s];
    }
    const float *lfac(const Clu &c, long s, long v) const { return c.lfac.data() + (v * segs.size() + s) * 2; }
};

bool read_exact(FILE *f, void *p, size_t n) { return std::fread(p, 1, n, f) == n; }

Index *load_index(const char *path) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return nullptr;
    auto idx = std::make_unique<Index>();
    uint64_t h[3];
    bool ok = read_exact(f, h, 24);
    if (ok) {
        idx->N = h[0];
        idx->D = h[1];
        idx->K = h[2];
        idx->centroids.resize(idx->K * idx->D);
        ok = read_exact(f, idx->centroids.data(), 4 * idx->centroids.size()) && read_exact(f, idx->qcfg, 32);
    }
    uint64_t nd = 0, nv = 0, ns = 0;
    ok = ok && read_exact(f, &nd, 8) && read_exact(f, &nv, 8);
    if (ok) {
        idx->var.resize(nv);
        ok = read_exact(f, idx->var.data(), 4 * nv) && read_exact(f, &ns, 8);
    }
    for (uint64_t s = 0; ok && s < ns; ++s) {
        uint64_t dp, b;
        uint8_t scfg[20], flag;
        ok = read_exact(f, &dp, 8) && read_exact(f, &b, 8) && read_exact(f, scfg, 20) && read_exact(f, &flag, 1);
        Seg sg{(long)dp, (long)b, {}};
        if (ok && flag) {
            sg.P.resize(dp * dp);
            ok = read_exact(f, sg.P.data(), 4 * dp * dp);
        }
        idx->segs.push_back(std::move(sg));
    }
    std::vector<uint64_t> sizes(idx->K);
    ok = ok && read_exact(f, sizes.data(), 8 * idx->K);
    if (ok) idx->derive();
    long S = (long)idx->segs.size();
    for (long c = 0; ok && c < idx->K; ++c) {
        Clu cl;
        cl.n = (long)sizes[c];
        cl.nb = (cl.n + kFS - 1) / kFS;
        if (S > 1) {
            cl.sfac.resize(64 * S * cl.nb);
            ok = read_exact(f, cl.sfac.data(), 4 * cl.sfac.size());
        }
        cl.scode.resize(idx->block_bytes * cl.nb);
        // compact multi-segment layouts index with 16-byte rounded segment arrays
        // (cluster_data.hpp:281-284) but save/load only long_stride * n bytes.
        long lc_alloc = idx->long_stride * cl.n;
        if (S > 1 && idx->compact) {
            long t = 0;
            for (long s = 0; s < S; ++s) t += (idx->long_pv[s] * cl.n + 15) / 16 * 16;
            lc_alloc = std::max(lc_alloc, t);
        }
        cl.lcode.assign(lc_alloc, 0);
        cl.lfac.resize(2 * S * cl.n);
        cl.ids.resize(cl.n);
        ok = ok && read_exact(f, cl.scode.data(), cl.scode.size()) &&
             read_exact(f, cl.lcode.data(), idx->long_stride * cl.n) &&
             read_exact(f, cl.lfac.data(), 4 * cl.lfac.size()) && read_exact(f, cl.ids.data(), 4 * cl.n);
        for (long s = 0; ok && s < S; ++s) {
            cl.cent.emplace_back(idx->segs[s].dim);
            ok = read_exact(f, cl.cent.back().data(), 4 * idx->segs[s].dim);
        }
        idx->clus.push_back(std::move(cl));
    }
    std::fclose(f);
    if (!ok) return nullptr;
    return idx.release();
}

// ResultPool (utils/pool.hpp:12-61), L2 only.
struct Pool {
    long cap, size = 0;
    std::vector<uint32_t> ids;
    std::vector<float> d;
    explicit Pool(long k) : cap(k), ids(k + 1, 0), d(k + 1, 0.0f) {}
    float distk() const { return size == cap ? d[size - 1] : std::numeric_limits<float>::max(); }
    void insert(uint32_t u, float dist) {
        if (size == cap && dist > d[size - 1]) return;
        long lo = 0, len = size;
        while (len > 1) {
            long half = len >> 1;
            len -= half;
            lo += (d[lo + half - 1] < dist) * half;
        }
        if (lo < size && d[lo] < dist) lo++;
        std::memmove(&ids[lo + 1], &ids[lo], (size - lo) * sizeof(uint32_t));
        ids[lo] = u;
        std::memmove(&d[lo + 1], &d[lo], (size - lo) * sizeof(float));
        d[lo] = dist;
        size += (size < cap);
    }
};

// Per-segment query state: CaqCluEstimator + Lut (caq_estimator.hpp:56-217, lut.hpp:60-126)
struct SegEst {
    long D = 0, bits = 0;
    std::vector<float> qrot;    // query_data_
    float prune = 0;            // without_ip_prune_bound_
    // per cluster
    std::vector<float> q;       // query_ = qrot - centroid
    std::vector<uint16_t> lut;  // D/4 x 16
    float delta = 0, sum_q = 0, sum_vl = 0, q_l2sqr = 0, q_l2norm = 0;
    float one_over_sqrtD = 0;
    float ipx[32];              // ip_xb_qprime_ of the current block

    void prepare(const float *cent) {
        q.resize(D);
        for (long i = 0; i < D; ++i) q[i] = qrot[i] - cent[i];
        sum_q = eigen_sum(q.data(), D);
        q_l2sqr = eigen_sqnorm(q.data(), D);
        q_l2norm = std::sqrt(q_l2sqr);
        const long ncb = D / 4;
        std::vector<float> lf(ncb * 16);
        for (long cb = 0; cb < ncb; ++cb) {
            float *t = &lf[cb * 16];
            t[0] = 0;
            for (int j = 1; j < 16; ++j) t[j] = t[j - (j & -j)] + q[cb * 4 + kPos[j]];
        }
        float vl = lf[0], vr = lf[0];
        for (float v : lf) {
            vl = std::min(vl, v);
            vr = std::max(vr, v);
        }
        delta = (float)((double)(vr - vl) / ((1 << 16) - 0.01));
        lut.resize(ncb * 16);
        for (long i = 0; i < ncb * 16; ++i) {
            float t = (lf[i] - vl) / delta;
            lut[i] = (uint16_t)(int32_t)t;
        }
        sum_vl = (float)((vl + 0.5 * delta) * (double)(float)ncb);
    }
    // compFastDist for one block; L2 (caq_estimator.hpp:148-179, lut.hpp:89-119)
    void fast(const uint8_t *blk, const float *onorm, float *out, int32_t *sums_out) {
        const long ncb = D / 4;
        const float c1 = (float)(0.5 * sum_q - (double)(0.58f * q_l2norm));
        const float c2 = 4 / 0.8f * one_over_sqrtD;
        for (int v = 0; v < 32; ++v) {
            int32_t s = 0;
            for (long cb = 0; cb < ncb; ++cb) s += lut[cb * 16 + block_nibble(blk, cb, v)];
            if (sums_out) sums_out[v] = s;
            float t = (float)s * delta;
            t = t + sum_vl;
            ipx[v] = t;
            float f = (t - c1) * c2;
            f = f * onorm[v];
            out[v] = maxps(0.0f, onorm[v] * onorm[v] + (q_l2sqr - f));
        }
    }
    void vars(const float *onorm, float *out) const {
        const float fv = q_l2sqr - 2 * prune;
        for (int v = 0; v < 32; ++v) out[v] = maxps(0.0f, onorm[v] * onorm[v] + fv);
    }
    float accurate(const float onorm, const uint8_t *lcode, const float *lfac, int j) const {
        const float o2 = onorm * onorm;
        if (bits == 0) return o2 + q_l2sqr;
        const float dl = (float)(2.0 / (1 << bits));
        double ex = excode_ip(q.data(), lcode, D, (int)bits - 1);
        float e = (float)((double)ipx[j] + ex * (double)dl + (-1.0 + (double)(dl / 2)) * (double)sum_q);
        float ipoq = lfac[0] * e;
        return o2 + q_l2sqr - 2 * ipoq;
    }
};

struct Query {
    const Index *idx;
    std::vector<SegEst> se;
    Query(const Index *ix, const float *query, float m) : idx(ix) {
        long off = 0;
        for (auto &sg : ix->segs) {
            SegEst e;
            e.D = sg.dim;
            e.bits = sg.bits;
            std::vector<float> cq(sg.dim, 0.0f);
            for (long i = 0; i < sg.dim && off + i < ix->D; ++i) cq[i] = query[off + i];
            float v2 = eigen_var_q2(ix->var.data() + off, cq.data(), sg.dim);
            e.prune = std::sqrt(v2) * m;
            e.qrot.resize(sg.dim);
            if (!sg.P.empty()) gemv_rowvec(cq.data(), sg.P.data(), sg.dim, e.qrot.data());
            else e.qrot = cq;
            e.one_over_sqrtD = (float)(1.0 / std::sqrt((float)sg.dim));
            se.push_back(std::move(e));
            off += sg.dim;
        }
    }
};

// FlatInitializer::centroids_distances (initializer.hpp:52-76)
struct Cand {
    uint32_t id;
    float distance;
    bool operator<(const Cand &o) const { return distance < o.distance; }
};
std::vector<Cand> probe(const Index *idx, const float *q, long nprobe) {
    std::vector<Cand> cd(idx->K);
    for (long i = 0; i < idx->K; ++i) {
        cd[i].id = (uint32_t)i;
        cd[i].distance = eigen_sqdist(idx->centroids.data() + i * idx->D, q, idx->D);
    }
    std::partial_sort(cd.begin(), cd.begin() + nprobe, cd.end());
    cd.resize(nprobe);
    return cd;
}

// SAQSearcher::searchCluster / scanCluster (saq_searcher.hpp:68-214)
void search_cluster(const Index *idx, Query &Q, long cid, Pool &pool) {
    const Clu &c = idx->clus[cid];
    const long S = (long)idx->segs.size();
    for (long s = 0; s < S; ++s) Q.se[s].prepare(c.cent[s].data());
    if (S == 1) {
        SegEst &e = Q.se[0];
        float distk = pool.distk();
        for (long b = 0; b < c.nb; ++b) {
            long cur = (b == c.nb - 1) ? c.n % kFS : kFS;
            float est[32];
            const float *on = idx->onorm(c, 0, b);
            if (e.bits == 0) e.vars(on, est);
            else e.fast(idx->codes(c, 0, b), on, est, nullptr);
            uint32_t mask = 0;
            for (int v = 0; v < 32; ++v) mask |= (uint32_t)(est[v] < distk) << v;
            mask &= (uint32_t)((1ull << cur) - 1);
            while (mask) {
                int j = __builtin_ctz(mask);
                mask &= mask - 1;
                long v = b * kFS + j;
                float d = e.accurate(on[j], idx->lcode(c, 0, v), idx->lfac(c, 0, v), j);
                pool.insert(c.ids[v], d);
                distk = pool.distk();
            }
        }
        return;
    }
    float distk = pool.distk();
    std::vector<float> cd(S * 32);
    for (long b = 0; b < c.nb; ++b) {
        float cur[32] = {0};
        for (long s = 0; s < S; ++s) {
            Q.se[s].vars(idx->onorm(c, s, b), &cd[s * 32]);
            for (int v = 0; v < 32; ++v) cur[v] = cur[v] + cd[s * 32 + v];
        }
        float mi = reduce_min32(cur);
        if (mi > distk) continue;
        for (long s = 0; s < S; ++s) {
            if (idx->segs[s].bits == 0) continue;
            for (int v = 0; v < 32; ++v) cur[v] = cur[v] - cd[s * 32 + v];
            Q.se[s].fast(idx->codes(c, s, b), idx->onorm(c, s, b), &cd[s * 32], nullptr);
            for (int v = 0; v < 32; ++v) cur[v] = cur[v] + cd[s * 32 + v];
            mi = reduce_min32(cur);
            if (mi > distk) break;
        }
        if (mi <= distk) {
            for (int j = 0; j < 32; ++j) {
                if (cur[j] < distk) {
                    long v = b * kFS + j;
                    if (v >= c.n) break;
                    float acc = cur[j];
                    for (long s = 0; s < S; ++s) {
                        acc += Q.se[s].accurate(idx->onorm(c, s, b)[j], idx->lcode(c, s, v), idx->lfac(c, s, v), j) -
                               cd[s * 32 + j];
                        if (acc >= distk) break;
                    }
                    pool.insert(c.ids[v], acc);
                    distk = pool.distk();
                }
            }
        }
    }
}

void search_one(const Index *idx, const float *q, long topk, long nprobe, float m, uint32_t *ids, float *dists) {
    auto cd = probe(idx, q, nprobe);
    Pool pool(topk);
    Query Q(idx, q, m);
    for (auto &c : cd) search_cluster(idx, Q, c.id, pool);
    std::memcpy(ids, pool.ids.data(), topk * sizeof(uint32_t));
    if (dists)
        for (long i = 0; i < topk; ++i) dists[i] = i < pool.size ? pool.d[i] : std::numeric_limits<float>::max();
}

// ------------------------------------------------------------------ build
void colwise_mean_var(const float *x, long N, long D, std::vector<float> &var) {
    // SaqDataMaker::compute_variance (saq_data.hpp:95-100).  data.colwise().mean()
    // is vectorised: Eigen packetwise_redux_impl (PartialReduxEvaluator.h:102-128),
    // x0 + ((x1+x2)+(x3+x4)) + ... per column; the variance's argument is a
    // rowwise() replicate expression without packet access, so its column sums
    // run sequentially.  Both are divided by the row count.
    auto colsum = [&](auto f, long col) {
        float p = f(0, col);
        long size4 = (N - 1) & ~3L;
        long i = 1;
        for (; i < size4; i += 4) p = p + ((f(i, col) + f(i + 1, col)) + (f(i + 2, col) + f(i + 3, col)));
        for (; i < N; ++i) p = p + f(i, col);
        return p;
    };
    std::vector<float> mean(D);
    for (long c = 0; c < D; ++c) mean[c] = colsum([&](long r, long cc) { return x[r * D + cc]; }, c) / (float)N;
    var.resize(D);
    for (long c = 0; c < D; ++c) {
        float p = 0.0f;
        for (long r = 0; r < N; ++r) {
            const float d = x[r * D + c] - mean[c];
            p = r == 0 ? d * d : p + d * d;
        }
        var[c] = p / (float)N;
    }
}


// ------------------------------------------------------------------ index build
// IVF::construct (ivf.hpp:130-184) -> IVF::save layout.  Rotation of every
// vector and centroid uses the GEMV order above (the reference's GEMM order for
// whole clusters depends on the host's cache-blocking sizes; its GEMV order is
// what it uses for the centroid and for single-vector clusters).
// fn(i) for i in [0, n) on `threads` threads, dynamically in chunks of 64.
template <class F>
void parallel_for(long n, int threads, F fn) {
    if (threads <= 1 || n < 128) {
        for (long i = 0; i < n; ++i) fn(i);
        return;
    }
    std::atomic<long> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t)
        th.emplace_back([&]() {
            for (long a; (a = next.fetch_add(64)) < n;)
                for (long i = a; i < std::min(n, a + 64); ++i) fn(i);
        });
    for (auto &t : th) t.join();
}

struct BuildCfg {
    float avg_bits;
    int seg, eqseg, rdlmt, rotate;
    float eps;
};

void put_cfg_bytes(const BuildCfg &c, uint8_t *q32, uint8_t *s20) {
    std::memset(q32, 0, 32);
    std::memset(s20, 0, 20);
    // QuantSingleConfig (config.h:12-19): quant_type, random_rotation, use_fastscan, rd_lmt, eps, ori_qB
    int32_t qt = 0, rd = c.rdlmt, ori = 0;
    std::memcpy(s20 + 0, &qt, 4);
    s20[4] = (uint8_t)(c.rotate != 0);
    s20[5] = 1;
    std::memcpy(s20 + 8, &rd, 4);
    std::memcpy(s20 + 12, &c.eps, 4);
    std::memcpy(s20 + 16, &ori, 4);
    // QuantizeConfig (config.h:21-27)
    int32_t eq = c.eqseg;
    std::memcpy(q32 + 0, &c.avg_bits, 4);
    std::memcpy(q32 + 4, &eq, 4);
    q32[8] = (uint8_t)(c.seg != 0);
    q32[9] = 0;
    std::memcpy(q32 + 12, s20, 20);
}

int build_index(const float *data, long N, long D, const float *cent, long K, const uint32_t *cids, const BuildCfg &cfg,
                const float *vars_in, const float *rots, const char *path, int threads) {
    if (D % 64) return 1;
    std::vector<float> var;
    if (vars_in) var.assign(vars_in, vars_in + D);
    else colwise_mean_var(data, N, D, var);
    Plan plan = !cfg.seg ? plan_equal(D, cfg.avg_bits, 1)
                         : (cfg.eqseg > 0 ? plan_equal(D, cfg.avg_bits, cfg.eqseg) : plan_dp(var.data(), D, cfg.avg_bits));
    const long S = (long)plan.segs.size();
    uint8_t q32[32], s20[20];
    put_cfg_bytes(cfg, q32, s20);
    std::vector<std::vector<uint32_t>> lists(K);
    for (long i = 0; i < N; ++i) lists[cids[i]].push_back((uint32_t)i);
    FILE *f = std::fopen(path, "wb");
    if (!f) return 2;
    auto w = [&](const void *p, size_t n) { std::fwrite(p, 1, n, f); };
    auto w64 = [&](uint64_t v) { w(&v, 8); };
    w64(N);
    w64(D);
    w64(K);
    w(cent, 4 * K * D);
    w(q32, 32);
    w64(D);
    w64(D);
    w(var.data(), 4 * D);
    w64(S);
    std::vector<long> roff(S, 0);
    long ro = 0;
    for (long s = 0; s < S; ++s) {
        const long d = plan.segs[s].first;
        w64(d);
        w64(plan.segs[s].second);
        w(s20, 20);
        uint8_t flag = cfg.rotate ? 1 : 0;
        w(&flag, 1);
        if (cfg.rotate) w(rots + ro, 4 * d * d);
        roff[s] = ro;
        ro += d * d;
    }
    for (long c = 0; c < K; ++c) w64(lists[c].size());
    Index meta;
    for (long s = 0; s < S; ++s) meta.segs.push_back(Seg{plan.segs[s].first, plan.segs[s].second, {}});
    std::memcpy(meta.qcfg, q32, 32);
    meta.derive();
    // Vectors in file order (cluster by cluster), cluster starts in vectors and in 32-vector blocks.
    std::vector<long> cstart(K + 1, 0), bstart(K + 1, 0), seg_off(S + 1, 0);
    for (long c = 0; c < K; ++c) {
        cstart[c + 1] = cstart[c] + (long)lists[c].size();
        bstart[c + 1] = bstart[c] + ((long)lists[c].size() + kFS - 1) / kFS;
    }
    for (long s = 0; s < S; ++s) seg_off[s + 1] = seg_off[s] + plan.segs[s].first;
    std::vector<uint32_t> order(N), clu_of(N);
    for (long c = 0; c < K; ++c)
        for (long v = 0; v < (long)lists[c].size(); ++v) {
            order[cstart[c] + v] = lists[c][v];
            clu_of[cstart[c] + v] = (uint32_t)c;
        }
    // Per-segment centroid slices (zero-padded) and their rotations.
    std::vector<std::vector<float>> cseg_all(K * S), rc_all(K * S);
    parallel_for(K, threads, [&](long c) {
        for (long s = 0; s < S; ++s) {
            const long d = plan.segs[s].first, off = seg_off[s];
            std::vector<float> &cs = cseg_all[c * S + s], &rc = rc_all[c * S + s];
            cs.assign(d, 0.0f);
            for (long i = 0; i < d && off + i < D; ++i) cs[i] = cent[c * D + off + i];
            rc.resize(d);
            if (cfg.rotate) gemv_rowvec(cs.data(), rots + roff[s], d, rc.data());
            else rc = cs;
        }
    });
    // Every vector encoded independently: factors, 1-bit codes (MSB-first bytes,
    // in block-padded slots) and ex-codes at their final places.
    const long nslots = bstart[K] * kFS;
    std::vector<float> onorm_all(N * S, 0.0f), ipco_all(N * S, 0.0f), lfac_all(2 * S * N, 0.0f);
    std::vector<std::vector<uint8_t>> shortc(S);
    for (long s = 0; s < S; ++s) shortc[s].assign(nslots * (plan.segs[s].first / 8), 0);
    std::vector<uint8_t> lc_all((size_t)meta.long_stride * N, 0);
    constexpr long kGroup = 8;  // vectors rotated together (one pass over P per group)
    parallel_for((N + kGroup - 1) / kGroup, threads, [&](long grp) {
        const long p0 = grp * kGroup, m = std::min(kGroup, N - p0);
        thread_local std::vector<float> xs, xr, o;
        thread_local std::vector<uint16_t> low;
        thread_local CaqOut out;
        for (long s = 0; s < S; ++s) {
            const long d = plan.segs[s].first, bits = plan.segs[s].second, off = seg_off[s];
            xs.assign((size_t)m * d, 0.0f);
            xr.resize((size_t)m * d);
            o.resize(d);
            for (long r = 0; r < m; ++r) {
                const float *x = data + (size_t)order[p0 + r] * D;
                for (long i = 0; i < d && off + i < D; ++i) xs[r * d + i] = x[off + i];
            }
            if (cfg.rotate) gemv_rows(xs.data(), m, rots + roff[s], d, xr.data());
            else xr = xs;
            for (long r = 0; r < m; ++r) {
                const long p = p0 + r, c = clu_of[p], v = p - cstart[c];
                const std::vector<float> &rc = rc_all[c * S + s];
                for (long i = 0; i < d; ++i) o[i] = xr[r * d + i] - rc[i];
                caq_encode(o.data(), d, (int)bits, cseg_all[c * S + s].data(), cfg.rdlmt, cfg.eps, out);
                onorm_all[p * S + s] = out.o_l2norm;
                if (bits == 0) continue;
                ipco_all[p * S + s] = out.ip_cent_oa;
                lfac_all[(p * S + s) * 2] = out.rescale;
                lfac_all[(p * S + s) * 2 + 1] = out.error;
                const int sb = 1 << (bits - 1);
                uint8_t *sc = &shortc[s][(size_t)(bstart[c] * kFS + v) * (d / 8)];
                for (long i = 0; i < d; ++i)
                    if (out.code[i] & sb) sc[i / 8] |= (uint8_t)(0x80 >> (i % 8));
                if (bits > 1) {
                    low.resize(d);
                    for (long i = 0; i < d; ++i) low[i] = (uint16_t)(out.code[i] & (sb - 1));
                    pack_excode(low.data(), d, (int)bits - 1,
                                lc_all.data() + (size_t)p * meta.long_stride + meta.long_off[s]);
                }
            }
        }
    });
    // Clusters in order: factor blocks and FastScan-packed 1-bit blocks, then the
    // per-vector arrays (IVF::save, ivf.hpp:197-233).
    for (long c = 0; c < K; ++c) {
        const long n = cstart[c + 1] - cstart[c], nb = bstart[c + 1] - bstart[c], p0 = cstart[c];
        std::vector<float> sfac(S > 1 ? 64 * S * nb : 0, 0.0f);
        std::vector<uint8_t> scode(meta.block_bytes * nb, 0);
        for (long v = 0; v < n; ++v) {
            const long b = v / kFS, j = v % kFS;
            for (long s = 0; s < S; ++s) {
                float *fac = S == 1 ? reinterpret_cast<float *>(scode.data() + b * meta.block_bytes)
                                    : sfac.data() + (b * S + s) * 64;
                fac[j] = onorm_all[(p0 + v) * S + s];
                if (plan.segs[s].second) fac[kFS + j] = ipco_all[(p0 + v) * S + s];
            }
        }
        for (long s = 0; s < S; ++s) {
            const long d = plan.segs[s].first;
            if (!plan.segs[s].second) continue;
            for (long b = 0; b < nb; ++b) {
                uint8_t *blk = S == 1 ? scode.data() + b * meta.block_bytes + 256 : scode.data() + b * meta.block_bytes + meta.sc_off[s];
                pack_block(&shortc[s][(size_t)(bstart[c] + b) * kFS * (d / 8)], d, blk);
            }
        }
        if (S > 1) w(sfac.data(), 4 * sfac.size());
        w(scode.data(), scode.size());
        w(lc_all.data() + (size_t)p0 * meta.long_stride, (size_t)n * meta.long_stride);
        w(lfac_all.data() + (size_t)p0 * 2 * S, 4 * (size_t)n * 2 * S);
        w(lists[c].data(), 4 * n);
        for (long s = 0; s < S; ++s) w(rc_all[c * S + s].data(), 4 * rc_all[c * S + s].size());
    }
    std::fclose(f);
    return 0;
}
}  // namespace

// ============================================================== C interface
extern "C" {

float orc_eigen_sum(const float *x, long n) { return eigen_sum(x, n); }
float orc_eigen_sqnorm(const float *x, long n) { return eigen_sqnorm(x, n); }
float orc_eigen_sqdist(const float *a, const float *b, long n) { return eigen_sqdist(a, b, n); }
void orc_gemv_rowvec(const float *q, const float *P, long D, float *out) { gemv_rowvec(q, P, D, out); }
float orc_excode_ip(const float *q, const uint8_t *code, long D, int ex_bits) { return excode_ip(q, code, D, ex_bits); }
void orc_pack_excode(const uint16_t *v, long D, int ex_bits, uint8_t *out) { pack_excode(v, D, ex_bits, out); }
void orc_unpack_excode(const uint8_t *y, long D, int ex_bits, uint16_t *out) { unpack_excode(y, D, ex_bits, out); }
void orc_pack_block(const uint8_t *sc, long D, uint8_t *blk) { pack_block(sc, D, blk); }
void orc_colwise_var(const float *x, long N, long D, float *var) {
    std::vector<float> v;
    colwise_mean_var(x, N, D, v);
    std::memcpy(var, v.data(), 4 * D);
}

int orc_plan(const float *var, long dpad, float avg_bits, int enable_seg, int eqseg, long *dims, long *bits, int cap) {
    Plan p = !enable_seg ? plan_equal(dpad, avg_bits, 1)
                         : (eqseg > 0 ? plan_equal(dpad, avg_bits, eqseg) : plan_dp(var, dpad, avg_bits));
    int n = (int)p.segs.size();
    for (int i = 0; i < n && i < cap; ++i) {
        dims[i] = p.segs[i].first;
        bits[i] = p.segs[i].second;
    }
    return n;
}

// facs: n x 4 (o_l2norm, ip_cent_oa, rescale, error)
int orc_caq_encode(const float *resid, long n, long D, int bits, const float *cent_unrot, int rdlmt, float eps,
                   int32_t *codes, float *facs) {
    CaqOut o;
    for (long i = 0; i < n; ++i) {
        caq_encode(resid + i * D, D, bits, cent_unrot, rdlmt, eps, o);
        for (long j = 0; j < D; ++j) codes[i * D + j] = o.code[j];
        facs[i * 4 + 0] = o.o_l2norm;
        facs[i * 4 + 1] = o.ip_cent_oa;
        facs[i * 4 + 2] = o.rescale;
        facs[i * 4 + 3] = o.error;
    }
    return 0;
}

void *orc_index_load(const char *path) { return load_index(path); }
void orc_index_free(void *h) { delete static_cast<Index *>(h); }
int orc_index_info(void *h, long *N, long *D, long *K, long *nseg) {
    auto *ix = static_cast<Index *>(h);
    *N = ix->N;
    *D = ix->D;
    *K = ix->K;
    *nseg = (long)ix->segs.size();
    return 0;
}

int orc_probe(void *h, const float *q, long nprobe, uint32_t *ids, float *d) {
    auto cd = probe(static_cast<Index *>(h), q, nprobe);
    for (long i = 0; i < nprobe; ++i) {
        ids[i] = cd[i].id;
        d[i] = cd[i].distance;
    }
    return 0;
}

// rotated query per segment (concatenated) and prune bounds
int orc_query_prep(void *h, const float *q, float m, float *rotq, float *prune) {
    auto *ix = static_cast<Index *>(h);
    Query Q(ix, q, m);
    long off = 0;
    for (size_t s = 0; s < Q.se.size(); ++s) {
        std::memcpy(rotq + off, Q.se[s].qrot.data(), 4 * Q.se[s].D);
        prune[s] = Q.se[s].prune;
        off += Q.se[s].D;
    }
    return 0;
}

// LUT of (query, cluster, segment): u16 table, scalars (delta, sum_vl, sum_q, q_l2sqr, q_l2norm),
// FastScan integer sums and fast distances for every block.
int orc_lut(void *h, const float *q, long cid, int seg, uint16_t *lut, float *scal, int32_t *sums, float *fast) {
    auto *ix = static_cast<Index *>(h);
    Query Q(ix, q, 4.0f);
    SegEst &e = Q.se[seg];
    const Clu &c = ix->clus[cid];
    e.prepare(c.cent[seg].data());
    std::memcpy(lut, e.lut.data(), 2 * e.lut.size());
    scal[0] = e.delta;
    scal[1] = e.sum_vl;
    scal[2] = e.sum_q;
    scal[3] = e.q_l2sqr;
    scal[4] = e.q_l2norm;
    if (e.bits)
        for (long b = 0; b < c.nb; ++b)
            e.fast(ix->codes(c, seg, b), ix->onorm(c, seg, b), fast + b * 32, sums + b * 32);
    return 0;
}

int orc_search(void *h, const float *q, long nq, long topk, long nprobe, float m, uint32_t *ids, float *dists,
               int threads) {
    auto *ix = static_cast<Index *>(h);
    if (threads <= 1) {
        for (long i = 0; i < nq; ++i)
            search_one(ix, q + i * ix->D, topk, nprobe, m, ids + i * topk, dists ? dists + i * topk : nullptr);
        return 0;
    }
    std::atomic<long> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t)
        th.emplace_back([&]() {
            for (long i; (i = next.fetch_add(1)) < nq;)
                search_one(ix, q + i * ix->D, topk, nprobe, m, ids + i * topk, dists ? dists + i * topk : nullptr);
        });
    for (auto &t : th) t.join();
    return 0;
}

// IVF::estimate (ivf.hpp:313-362) for one query; returns the number of vectors written.
long orc_estimate(void *h, const float *q, long nprobe, float m, uint32_t *ids, float *acc, float *fast, float *vars,
                  long cap) {
    auto *ix = static_cast<Index *>(h);
    auto cd = probe(ix, q, nprobe);
    Query Q(ix, q, m);
    const long S = (long)ix->segs.size();
    long w = 0;
    for (auto &cc : cd) {
        const Clu &c = ix->clus[cc.id];
        for (long s = 0; s < S; ++s) Q.se[s].prepare(c.cent[s].data());
        for (long b = 0; b < c.nb; ++b) {
            float fsum[32] = {0}, vsum[32] = {0}, t[32];
            for (long s = 0; s < S; ++s) {
                if (Q.se[s].bits == 0) Q.se[s].vars(ix->onorm(c, s, b), t);
                else Q.se[s].fast(ix->codes(c, s, b), ix->onorm(c, s, b), t, nullptr);
                for (int v = 0; v < 32; ++v) fsum[v] = fsum[v] + t[v];
                Q.se[s].vars(ix->onorm(c, s, b), t);
                for (int v = 0; v < 32; ++v) vsum[v] = vsum[v] + t[v];
            }
            for (int j = 0; j < 32 && b * kFS + j < c.n; ++j) {
                long v = b * kFS + j;
                float a = 0;
                for (long s = 0; s < S; ++s)
                    a += Q.se[s].accurate(ix->onorm(c, s, b)[j], ix->lcode(c, s, v), ix->lfac(c, s, v), j);
                if (w < cap) {
                    ids[w] = c.ids[v];
                    acc[w] = a;
                    fast[w] = fsum[j];
                    vars[w] = vsum[j];
                }
                ++w;
            }
        }
    }
    return w;
}

// Model of the tensor-core form's approximate distance (the reference has no
// such form): per segment |o|^2 + |r|^2 - 2 rescale (delta <r, u> + (delta/2 - 1) sum r),
// r the rotated residual query, u the full B-bit code ((1-bit code << (B-1)) |
// ex-code), delta = 2 / 2^B, all in double; for every vector of the probed
// clusters in the order of orc_estimate.  It is CaqCluEstimator::compAccurateDist
// (caq_estimator.hpp:190-217) with the 1-bit part's u16 LUT replaced by the
// exact code.
long orc_tc_approx(void *h, const float *q, long nprobe, float m, uint32_t *ids, double *approx, long cap) {
    auto *ix = static_cast<Index *>(h);
    auto cd = probe(ix, q, nprobe);
    Query Q(ix, q, m);
    const long S = (long)ix->segs.size();
    long w = 0;
    std::vector<uint16_t> ex;
    for (auto &cc : cd) {
        const Clu &c = ix->clus[cc.id];
        for (long s = 0; s < S; ++s) Q.se[s].prepare(c.cent[s].data());
        for (long v = 0; v < c.n; ++v) {
            const long b = v / kFS;
            const int j = (int)(v % kFS);
            double a = 0;
            for (long s = 0; s < S; ++s) {
                const SegEst &e = Q.se[s];
                const double on = ix->onorm(c, s, b)[j];
                double sq = 0, sr = 0, ip = 0;
                for (long d = 0; d < e.D; ++d) {
                    sq += (double)e.q[d] * e.q[d];
                    sr += e.q[d];
                }
                if (e.bits == 0) {
                    a += on * on + sq;
                    continue;
                }
                ex.assign(e.D, 0);
                if (e.bits > 1) unpack_excode(ix->lcode(c, s, v), e.D, (int)e.bits - 1, ex.data());
                const uint8_t *blk = ix->codes(c, s, b);
                for (long d = 0; d < e.D; ++d) {
                    const long msb = (block_nibble(blk, d / 4, j) >> (3 - d % 4)) & 1;
                    ip += (double)((msb << (e.bits - 1)) | ex[d]) * e.q[d];
                }
                const double dl = 2.0 / (double)(1L << e.bits);
                a += on * on + sq - 2.0 * ix->lfac(c, s, v)[0] * (dl * ip + (dl / 2 - 1.0) * sr);
            }
            if (w < cap) {
                ids[w] = c.ids[v];
                approx[w] = a;
            }
            ++w;
        }
    }
    return w;
}

// threads <= 0: every hardware thread.  The file does not depend on the thread count.
int orc_build_index(const float *data, long N, long D, const float *cent, long K, const uint32_t *cids, float avg_bits,
                    int seg, int eqseg, int rdlmt, float eps, int rotate, const float *vars, const float *rots,
                    const char *path, int threads) {
    BuildCfg c{avg_bits, seg, eqseg, rdlmt, rotate, eps};
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    return build_index(data, N, D, cent, K, cids, c, vars, rots, path, threads);
}

}  // extern "C"
