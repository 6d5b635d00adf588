// Float-float pieces of the order-2 refinement step of the derivative sweep
// (k_grad<DIM, 2, NF, true> in mg_grad.cu).  Host and device: the CPU tests
// compile this header into a host program and check it against FP64.
#pragma once
#include <math.h>

#include "mg_common.cuh"

namespace mg {

// Rounded product that the compiler may not fuse into a following add (its
// FMA error term is taken separately).
__host__ __device__ __forceinline__ float mul_rn(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    volatile float p = a * b;
    return p;
#endif
}

// Separation component from the hi/lo split with its rounding error: returns
// exactly what sep_hilo computes for that component, and lo such that
// return + lo is the separation to ~2^-48 of the positions' magnitude (TwoSum
// on both steps; only the difference of the two low parts rounds, at 2^-24 of
// itself).
__host__ __device__ __forceinline__ float sep1_ff(float hb, float ha, float lb, float la, float &lo) {
    float s, e, d, e2;
    two_sum(hb, -ha, s, e);
    two_sum(s, lb - la, d, e2);
    lo = e2 + e;
    return d;
}

// wrap1 (the nearest-image separation) with its rounding error, as sep1_ff.
__host__ __device__ __forceinline__ float wrap1_ff(float hb, float ha, float lb, float la, float box_hi,
                                                   float box_lo, float &lo) {
    float s, e;
    two_sum(hb, -ha, s, e);
    const float l = lb - la;
    const float d = s + (e + l);
    float r, er;
    if (fabsf(d) > 0.5f * box_hi) {
        const float sg = d > 0.0f ? 1.0f : -1.0f;
        float s2, e2;
        two_sum(s, -sg * box_hi, s2, e2);
        two_sum(s2, (e2 + e + l) - sg * box_lo, r, er);
    } else {
        two_sum(s, e + l, r, er);
    }
    lo = er;
    return r;
}

// Low part of the scaled separation: with x = d * hinv rounded, x + the
// return value is (d + dlo) * hinv to ~2^-48 (the FMA error of the scaling
// plus the separation's own rounding error).
__host__ __device__ __forceinline__ float scaled_sep_lo(float d, float dlo, float hinv, float x) {
    return fmaf(d, hinv, -x) + dlo * hinv;
}

// A separation scaled by 1/h given as a float-float pair (hh + hl): rounded
// once, so the scaling itself is carried to ~2^-46 for the whole row.
__host__ __device__ __forceinline__ float scale_sep(float d, float hh, float hl) { return fmaf(d, hl, d * hh); }

// Low part of a separation (d + dlo) scaled by (hh + hl), x = scale_sep(d,
// hh, hl): x + the return value is the product to ~2^-46.
__host__ __device__ __forceinline__ float scaled_sep_lo2(float d, float dlo, float hh, float hl, float x) {
    return fmaf(d, hh, -x) + fmaf(d, hl, dlo * hh);
}

// Residual of one neighbour and one component for the refinement step,
// e = (f_j - f_i) - a . sol: the field difference from the hi/lo splits and
// the linear part of the prediction, (x + xl) . sol[0:DIM], as float-float
// pairs, so that the large first-derivative part cancels exactly; the
// quadratic part a[DIM:ND] . sol[DIM:ND] in FP32.  a is the FP32 basis at x.
template <int DIM, int ND>
__host__ __device__ __forceinline__ float refine_residual(const float x[3], const float xl[3], const float *a,
                                                          const float *sol, float fh, float fl, float f0h,
                                                          float f0l) {
    float sh = 0.0f, sl = 0.0f;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const float p = mul_rn(x[d], sol[d]);
        const float pe = fmaf(x[d], sol[d], -p);
        float t, te;
        two_sum(sh, p, t, te);
        sh = t;
        sl += (te + pe) + xl[d] * sol[d];
    }
    float quad = 0.0f;
#pragma unroll
    for (int m = DIM; m < ND; ++m) quad = fmaf(a[m], sol[m], quad);
    float dh, de;
    two_sum(fh, -f0h, dh, de);
    const float dlf = (fl - f0l) + de;
    return ((dh - sh) + (dlf - sl)) - quad;
}

}  // namespace mg
