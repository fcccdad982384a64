// Segment bit planner: SaqDataMaker::analyze_plan (quantization/saq_data.hpp:119-227).
//
// Dynamic program over 64-dimension blocks: f[ns][i][bits] = least sum over
// segments of var_sum(segment) / 2^b, using ns segments to cover the first i
// blocks with `bits` total bits (64 bits of short factors charged per segment).
// A 0-bit tail segment may close the plan.  The result keeps the reference's
// tie rules: an end state replaces the current answer only if it is 1 % better,
// transitions replace only on strict improvement, and states are visited in
// (ns, i, bits) order.  Block variance sums use Eigen's 16-lane float order.
#include <algorithm>
#include <cstdint>
#include <limits>
#include <vector>

#include "saqg_internal.h"

namespace saqg {

namespace {
float eigen_sum64(const float *x) {
    // Redux.h:227-283 for 64 floats: accumulators over packets {0,2} and {1,3}
    float r0[16], r1[16];
    for (int l = 0; l < 16; ++l) {
        r0[l] = x[l] + x[32 + l];
        r1[l] = x[16 + l] + x[48 + l];
        r0[l] = r0[l] + r1[l];
    }
    float a[8], b[4];
    for (int i = 0; i < 8; ++i) a[i] = r0[i] + r0[i + 8];
    for (int i = 0; i < 4; ++i) b[i] = a[i] + a[i + 4];
    return (b[0] + b[2]) + (b[1] + b[3]);
}
}  // namespace

std::vector<std::pair<int64_t, int64_t>> make_plan(const float *var, int64_t Dp, float avg_bits, bool seg, int eqseg) {
    std::vector<std::pair<int64_t, int64_t>> plan;
    if (!seg || eqseg > 0) {  // equal_segmentation (saq_data.hpp:133-145)
        const int nseg = seg ? eqseg : 1;
        const int64_t b = (int64_t)avg_bits;
        int64_t d = 0;
        for (int i = 0; i < nseg && d < Dp; i++) {
            const int64_t t = ((Dp - d) / (nseg - i) + 63) / 64 * 64;
            plan.emplace_back(t, b);
            d += t;
        }
        return plan;
    }
    const size_t nbf = 2 * sizeof(float) * 8;
    const size_t tot_bits = (size_t)(avg_bits * (float)Dp + (float)nbf);
    const size_t max_ns = avg_bits < 2 ? Dp / 64 : Dp / 64 / 2;
    const size_t i_end = Dp / 64, W = tot_bits + 1, H = i_end + 1;
    const double lim = std::numeric_limits<double>::max();
    std::vector<double> fv((max_ns + 1) * H * W, lim);
    std::vector<uint32_t> fs((max_ns + 1) * H * W, 0);
    auto at = [&](size_t ns, size_t i, size_t b) { return (ns * H + i) * W + b; };
    std::vector<float> blk(i_end);
    for (size_t i = 0; i < i_end; ++i) blk[i] = eigen_sum64(var + 64 * i);
    size_t ans_ns = 0, ans_i = i_end, ans_b = tot_bits;
    fv[at(0, 0, 0)] = 0;
    for (size_t ns = 0; ns <= max_ns; ns++)
        for (size_t i = 0; i <= i_end; i++)
            for (size_t ub = 0; ub <= tot_bits; ++ub) {
                const double cur = fv[at(ns, i, ub)];
                if (!(cur < lim)) continue;
                if (i == i_end) {
                    if (cur * 1.01 < fv[at(ans_ns, ans_i, ans_b)]) {
                        ans_ns = ns;
                        ans_i = i;
                        ans_b = ub;
                    }
                    continue;
                }
                if (ns == max_ns) continue;
                double var_sum = 0;
                for (size_t j = 1; (i + j) * 64 <= (size_t)Dp; j++) {
                    var_sum += blk[i + j - 1];
                    for (size_t b = 1; b <= (size_t)kMaxBits; ++b) {
                        const size_t Bn = ub + b * j * 64 + nbf;
                        if (Bn > tot_bits) break;
                        const double v = var_sum / (1 << b);
                        const size_t t = at(ns + 1, i + j, Bn);
                        if (fv[t] > cur + v) {
                            fv[t] = cur + v;
                            fs[t] = (uint32_t)((i << 4) + b);
                        }
                    }
                }
                const size_t t = at(ns + 1, i_end, ub);
                if (cur + var_sum < fv[t]) {
                    fv[t] = cur + var_sum;
                    fs[t] = (uint32_t)(i << 4);
                }
            }
    size_t ns = ans_ns, i = ans_i, B = ans_b;
    while (i > 0) {
        const uint32_t s = fs[at(ns, i, B)];
        const size_t pi = s >> 4, bits = s & 0xf, len = (i - pi) * 64;
        plan.emplace_back((int64_t)len, (int64_t)bits);
        ns--;
        i = pi;
        if (bits) B -= bits * len + nbf;
    }
    std::reverse(plan.begin(), plan.end());
    return plan;
}

}  // namespace saqg
