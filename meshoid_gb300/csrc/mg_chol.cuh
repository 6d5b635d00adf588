// FP32 Cholesky factor, solve and condition estimate of the packed
// symmetric moment matrices of the derivative sweep (k_grad in mg_grad.cu).
// Host and device: the CPU tests build this header into a host program that
// checks it against FP64.
#pragma once
#include <math.h>

#include "mg_common.cuh"

namespace mg {

// In-place FP32 Cholesky of a packed symmetric matrix (row-major lower
// triangle: index i*(i+1)/2 + j).  Returns false on a non-positive pivot
// (which is then replaced by 1 so the rest of the factor stays finite).
// Every loop has a constant trip count with the triangular bounds as
// compile-time guards and there is no early exit, so after unrolling every
// index is a constant and the factor stays in registers (loops bounded by an
// outer index, or a return from inside them, left it in local memory).
template <int N>
__host__ __device__ __forceinline__ bool cholesky(float m[N * (N + 1) / 2]) {
    bool ok = true;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        float s = m[j * (j + 1) / 2 + j];
#pragma unroll
        for (int p = 0; p < N; ++p)
            if (p < j) s -= m[j * (j + 1) / 2 + p] * m[j * (j + 1) / 2 + p];
        const bool pos = s > 0.0f;
        ok = ok && pos;
        const float d = sqrtf(pos ? s : 1.0f);
        m[j * (j + 1) / 2 + j] = d;
        const float inv = 1.0f / d;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            if (i > j) {
                float t = m[i * (i + 1) / 2 + j];
#pragma unroll
                for (int p = 0; p < N; ++p)
                    if (p < j) t -= m[i * (i + 1) / 2 + p] * m[j * (j + 1) / 2 + p];
                m[i * (i + 1) / 2 + j] = t * inv;
            }
        }
    }
    return ok;
}

// The same (kept as a separate name for callers that read better with it).
template <int N>
__host__ __device__ __forceinline__ bool cholesky_nb(float m[N * (N + 1) / 2]) {
    return cholesky<N>(m);
}

template <int N>
__host__ __device__ __forceinline__ void chol_solve(const float m[N * (N + 1) / 2], float b[N]) {
#pragma unroll
    for (int i = 0; i < N; ++i) {
        float t = b[i];
#pragma unroll
        for (int p = 0; p < N; ++p)
            if (p < i) t -= m[i * (i + 1) / 2 + p] * b[p];
        b[i] = t / m[i * (i + 1) / 2 + i];
    }
#pragma unroll
    for (int ii = 0; ii < N; ++ii) {
        const int i = N - 1 - ii;
        float t = b[i];
#pragma unroll
        for (int p = 0; p < N; ++p)
            if (p > i) t -= m[p * (p + 1) / 2 + i] * b[p];
        b[i] = t / m[i * (i + 1) / 2 + i];
    }
}

// Condition-number estimate of the packed symmetric M (Cholesky factor L).
// 1x1: 1.  2x2 and 3x3: exact eigenvalues (closed form).  Larger: the upper
// bound trace(M) * trace(M^-1), with trace(M^-1) = sum of squared entries of
// L^-1.
template <int N>
__host__ __device__ __forceinline__ float cond_estimate(const float m[N * (N + 1) / 2], const float l[N * (N + 1) / 2]) {
    if (N == 1) return 1.0f;
    if (N == 2) {
        const float a = m[0], b = m[1], c = m[2];
        const float mean = 0.5f * (a + c), d = sqrtf(0.25f * (a - c) * (a - c) + b * b);
        const float lo = mean - d;
        return lo > 0.0f ? (mean + d) / lo : 1e30f;
    }
    if (N == 3) {
        // Smith (1961): eigenvalues of a symmetric 3x3 from its invariants
        const float a00 = m[0], a10 = m[1], a11 = m[2], a20 = m[3], a21 = m[4], a22 = m[5];
        const float q = (a00 + a11 + a22) / 3.0f;
        const float p1 = a10 * a10 + a20 * a20 + a21 * a21;
        const float b00 = a00 - q, b11 = a11 - q, b22 = a22 - q;
        const float p2 = b00 * b00 + b11 * b11 + b22 * b22 + 2.0f * p1;
        const float pp = sqrtf(p2 / 6.0f);
        if (!(pp > 0.0f)) return 1.0f;
        const float ip = 1.0f / pp;
        const float c00 = b00 * ip, c11 = b11 * ip, c22 = b22 * ip, c10 = a10 * ip, c20 = a20 * ip, c21 = a21 * ip;
        float r = 0.5f * (c00 * (c11 * c22 - c21 * c21) - c10 * (c10 * c22 - c21 * c20) + c20 * (c10 * c21 - c11 * c20));
        r = fminf(1.0f, fmaxf(-1.0f, r));
        const float phi = acosf(r) / 3.0f;
        // phi and phi + 2 pi / 3 lie in [0, pi]: the device's fast cosine
        // (no large-argument reduction path, whose scratch array put a stack
        // frame on every kernel that includes this estimate) is ample for a
        // condition estimate
#ifdef __CUDA_ARCH__
        const float e1 = q + 2.0f * pp * __cosf(phi);
        const float e3 = q + 2.0f * pp * __cosf(phi + 2.0943951023931953f);
#else
        const float e1 = q + 2.0f * pp * cosf(phi);
        const float e3 = q + 2.0f * pp * cosf(phi + 2.0943951023931953f);
#endif
        return e3 > 0.0f ? e1 / e3 : 1e30f;
    }
    float tr = 0.0f, tri = 0.0f;
#pragma unroll
    for (int i = 0; i < N; ++i) tr += m[i * (i + 1) / 2 + i];
    // columns of L^-1 by forward substitution on unit vectors
#pragma unroll
    for (int c = 0; c < N; ++c) {
        float x[N];
#pragma unroll
        for (int i = 0; i < N; ++i) {
            float t = (i == c) ? 1.0f : 0.0f;
#pragma unroll
            for (int p = 0; p < N; ++p)
                if (p < i) t -= l[i * (i + 1) / 2 + p] * x[p];
            x[i] = (i < c) ? 0.0f : t / l[i * (i + 1) / 2 + i];
            tri += x[i] * x[i];
        }
    }
    return tr * tri;
}

}  // namespace mg
