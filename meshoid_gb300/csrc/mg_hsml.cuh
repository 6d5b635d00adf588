// Smoothing length from a query's k neighbour distances (HsmlIter,
// src/meshoid/kernel_density.py:15-56), host and device: the search kernels
// call it per query, and the CPU tests build it into a host program that
// checks it against an FP64 bisection.
#pragma once
#include <float.h>
#include <math.h>

#include "mg_common.cuh"

// MG_HSML_COMPENSATED 1 (the default) sums n = norm sum_j W(d_j / h) with
// Kahan compensation: the FP32 rounding of that sum is what limits h where
// n's slope in h is small (1-D rows whose distances span decades: 1.25e-6
// relative error with a plain sum, 4.7e-7 compensated), and it keeps
// equal-distance rows from running to the iteration cap.  It costs three
// FP32 adds per neighbour and Newton step.  0 gives the plain sum.
#ifndef MG_HSML_COMPENSATED
#define MG_HSML_COMPENSATED 1
#endif

namespace mg {

// norm * sum_j W(d_j / h) = k over the query's k neighbour distances, by
// bracketed Newton with bisection fallback.  Bracket as the reference:
// [second-smallest distance, largest * bound_coeff]; first guess the largest
// distance (h is within ~10% of it for a smooth density).  Stops one Newton
// step after |n - k| <= 1e-6 k.  dist(j) returns the j-th distance (not
// squared).  lo_out (optional): the last Newton step is kept as an
// unevaluated sum, h + *lo_out = the previous iterate + the step exactly
// (TwoSum), which carries the root past the FP32 rounding of h (~3e-8) to
// the noise floor of the compensated neighbour count, ~1e-8 relative; 0 when
// the last step was a bisection.  FF: a float-float Newton step follows
// (hsml_polish_ff), which needs h within ~1e-6; the solve then also stops at
// the first close iterate whose Newton step is at most 1e-5 h (the next
// iterate is then ~1e-10 off) instead of taking one more step.
template <int DIM, int KU, bool FF = false, class Dist>
__host__ __device__ __forceinline__ float hsml_newton(Dist dist, int k, int &it, float *lo_out = nullptr) {
    const float norm = DIM == 3 ? 32.0f / 3.0f : (DIM == 2 ? 40.0f / 7.0f : 8.0f / 3.0f);
    const float bound_coeff = 1.0f / (1.0f - powf(2.0f * norm, -1.0f / 3.0f));
    float m1 = FLT_MAX, m2 = FLT_MAX, dmax = 0.0f;
#pragma unroll
    for (int j = 0; j < (KU > 0 ? KU : k); ++j) {
        if (KU > 0 && j >= k) break;
        const float d = dist(j);
        dmax = fmaxf(dmax, d);
        if (d < m1) {
            m2 = m1;
            m1 = d;
        } else if (d < m2) {
            m2 = d;
        }
    }
    float lower = m2, upper = dmax * bound_coeff;
    float h = dmax;
    if (!(h > lower && h < upper)) h = 0.5f * (lower + upper);
    const float kf = (float)k;
    bool polish = false;
    for (; it < 60; ++it) {
        const float hinv = 1.0f / h;
        float sw = 0.0f, sdw = 0.0f;
#if MG_HSML_COMPENSATED
        float cw = 0.0f;
#endif
#pragma unroll
        for (int j = 0; j < (KU > 0 ? KU : k); ++j) {
            if (KU > 0 && j >= k) break;
            const float qq = dist(j) * hinv;
#if MG_HSML_COMPENSATED
            const float y = spline_w(qq) - cw;
            const float t = sw + y;
            cw = (t - sw) - y;
            sw = t;
#else
            sw += spline_w(qq);
#endif
            sdw += spline_dw(qq) * qq;
        }
        const float F = norm * sw - kf;
        const float dF = -norm * sdw * hinv;  // dn/dh >= 0
        const bool close = fabsf(F) <= 1e-6f * kf;
        if (F > 0.0f)
            upper = h;
        else
            lower = h;
        const float step = (dF > 0.0f) ? -F / dF : 0.0f;
        float hn = (dF > 0.0f) ? h + step : -1.0f;
        const bool newton = hn >= lower && hn <= upper;
        if (!newton) hn = 0.5f * (lower + upper);
        const bool done = polish || fabsf(hn - h) <= 1e-8f * h || (upper - lower) <= 1e-8f * h ||
                          (FF && close && newton && fabsf(hn - h) <= 1e-5f * h);
        if (done && lo_out) {
            float s = hn, e = 0.0f;
            if (newton) two_sum(h, step, s, e);
            hn = s;
            *lo_out = e;
        }
        h = hn;
        if (done) break;
        polish = close;
    }
    return h;
}

}  // namespace mg
