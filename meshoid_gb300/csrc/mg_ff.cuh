// Float-float arithmetic (a value carried as an unevaluated sum hi + lo of two
// FP32 numbers, ~2^-44 relative) for the order-2 derivative sweep, host and
// device.  The CPU tests build this header, with the per-row routine of
// mg_grad2.cuh, into a host program and compare it with FP64.
//
// Error-free transformations used (Dekker 1971, Knuth TAOCP vol. 2 4.2.2):
//   TwoSum(a, b)      = (s, e) with s = fl(a + b) and s + e = a + b exactly;
//   TwoProd(a, b)     = (p, e) with p = fl(a * b) and e = fma(a, b, -p), exact.
// Products and sums whose error term is taken separately are computed with
// round-to-nearest intrinsics so that the compiler cannot contract them into
// a following FMA (which would change the rounded value the error term
// describes).
#pragma once
#include <math.h>

namespace mg {

struct ff {
    float hi, lo;
};

__host__ __device__ __forceinline__ float ff_mul_rn(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    volatile float p = a * b;
    return p;
#endif
}

__host__ __device__ __forceinline__ float ff_add_rn(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    volatile float s = a + b;
    return s;
#endif
}

__host__ __device__ __forceinline__ ff ff_make(float hi, float lo = 0.0f) { return ff{hi, lo}; }

// s + e = a + b exactly
__host__ __device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = ff_add_rn(a, b);
    const float bb = ff_add_rn(s, -a);
    const float e = ff_add_rn(ff_add_rn(a, -ff_add_rn(s, -bb)), ff_add_rn(b, -bb));
    return ff{s, e};
}

// |a| >= |b| (or a == 0): s + e = a + b exactly
__host__ __device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {
    const float s = ff_add_rn(a, b);
    return ff{s, ff_add_rn(b, -ff_add_rn(s, -a))};
}

__host__ __device__ __forceinline__ ff ff_norm(ff a) { return ff_fast_two_sum(a.hi, a.lo); }

__host__ __device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = ff_two_sum(a.hi, b.hi);
    s.lo = ff_add_rn(s.lo, ff_add_rn(a.lo, b.lo));
    return ff_norm(s);
}

__host__ __device__ __forceinline__ ff ff_add_f(ff a, float b) {
    ff s = ff_two_sum(a.hi, b);
    s.lo = ff_add_rn(s.lo, a.lo);
    return ff_norm(s);
}

__host__ __device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }

// product, normalised; the lo * lo term (2^-48 relative) is dropped
__host__ __device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = ff_mul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return ff_fast_two_sum(p, e);
}

__host__ __device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    const float p = ff_mul_rn(a.hi, b);
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return ff_fast_two_sum(p, e);
}

__host__ __device__ __forceinline__ ff ff_sqr(ff a) {
    const float p = ff_mul_rn(a.hi, a.hi);
    float e = fmaf(a.hi, a.hi, -p);
    e = fmaf(2.0f * a.hi, a.lo, e);
    return ff_fast_two_sum(p, e);
}

// sqrt by one Newton correction of an approximate root, with no division:
// y ~ 1/sqrt(a), s = a y ~ sqrt(a) (a few ulps off), then
// s + (a - s^2) y / 2, the residual a - s^2 exact by FMA.  The correction is
// ~1e-7 of s, so y's own ~1e-7 error leaves ~1e-14 of the result.
__host__ __device__ __forceinline__ ff ff_sqrt(ff a) {
    if (!(a.hi > 0.0f)) return ff{0.0f, 0.0f};
#ifdef __CUDA_ARCH__
    const float y = rsqrtf(a.hi);
#else
    const float y = 1.0f / sqrtf(a.hi);
#endif
    const float s = a.hi * y;
    const float r = ff_add_rn(fmaf(-s, s, a.hi), a.lo);
    return ff_fast_two_sum(s, r * (0.5f * y));
}

// 1 / b for an FP32 b, as a float-float pair
__host__ __device__ __forceinline__ ff ff_recip(float b) {
    const float r = 1.0f / b;
    return ff_fast_two_sum(r, fmaf(-b, r, 1.0f) * r);
}

// Accumulator: acc += p with the error of the addition carried in acc.lo,
// left unnormalised (at most a few tens of terms are summed, so acc.lo stays
// within a few ulps of acc.hi); ff_norm it before use.
__host__ __device__ __forceinline__ void ff_acc(ff &acc, ff p) {
    const ff s = ff_two_sum(acc.hi, p.hi);
    acc.hi = s.hi;
    acc.lo = ff_add_rn(acc.lo, ff_add_rn(s.lo, p.lo));
}

// acc += a * b for float-float a and b (product error included)
__host__ __device__ __forceinline__ void ff_fma_acc(ff &acc, ff a, ff b) {
    const float p = ff_mul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    const ff s = ff_two_sum(acc.hi, p);
    acc.hi = s.hi;
    acc.lo = ff_add_rn(acc.lo, ff_add_rn(s.lo, e));
}

// acc += a * b for float-float a and FP32 b
__host__ __device__ __forceinline__ void ff_fma_acc_f(ff &acc, ff a, float b) {
    const float p = ff_mul_rn(a.hi, b);
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    const ff s = ff_two_sum(acc.hi, p);
    acc.hi = s.hi;
    acc.lo = ff_add_rn(acc.lo, ff_add_rn(s.lo, e));
}

__host__ __device__ __forceinline__ float ff_to_f(ff a) { return a.hi + a.lo; }

// 1 / (hi + lo) as a float-float pair (hi + lo normalised, hi > 0)
__host__ __device__ __forceinline__ ff ff_recip2(float hi, float lo) {
    const float r = 1.0f / hi;
    const float e = fmaf(-hi, r, 1.0f) - lo * r;  // 1 - (hi + lo) r, to first order
    return ff_fast_two_sum(r, e * r);
}

// p / q for small integers p, q (exact in FP32) as a float-float pair
__host__ __device__ __forceinline__ ff ff_ratio(float p, float q) {
    const float r = p / q;
    return ff_fast_two_sum(r, fmaf(-q, r, p) / q);
}

// f_j - f_i from three-plane splits f = hi + mid + lo (each plane the FP32
// rounding of what the previous planes leave, so the split carries ~2^-72 of
// |f|): the difference is carried to ~2^-48 of itself plus 2^-72 of |f|,
// where a two-plane split would leave 2^-48 of |f| -- too coarse for
// neighbours whose values agree to many digits.
__host__ __device__ __forceinline__ ff ff_diff3(float hj, float mj, float lj, float hi, float mi, float li) {
    const ff s = ff_two_sum(hj, -hi);
    const ff t = ff_two_sum(mj, -mi);
    const ff v = ff_two_sum(s.hi, t.hi);
    const float lo = ff_add_rn(ff_add_rn(ff_add_rn(s.lo, t.lo), v.lo), ff_add_rn(lj, -li));
    return ff_fast_two_sum(v.hi, lo);
}

// Cubic spline W(q) of src/meshoid/kernel_density.py:82-96 in float-float,
// from q and q^2: 1 - 6 q^2 + 6 q^3 = 1 + q^2 (6 q - 6) for q <= 1/2,
// 2 (1 - q)^3 for 1/2 < q <= 1, 0 beyond.
__host__ __device__ __forceinline__ ff ff_spline_w(ff q, ff q2) {
    if (q.hi > 1.0f || (q.hi == 1.0f && q.lo >= 0.0f)) return ff{0.0f, 0.0f};
    if (q.hi < 0.5f || (q.hi == 0.5f && q.lo <= 0.0f)) {
        const ff t = ff_add_f(ff_mul_f(q, 6.0f), -6.0f);
        return ff_add_f(ff_mul(q2, t), 1.0f);
    }
    const ff a = ff_add_f(ff_neg(q), 1.0f);
    const ff a3 = ff_mul(ff_sqr(a), a);
    return ff{2.0f * a3.hi, 2.0f * a3.lo};
}

}  // namespace mg
