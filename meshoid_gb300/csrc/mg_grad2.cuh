// Order-2 least-squares derivatives in float-float, host and device: the
// kernels of mg_grad2.cu run these per query thread, and the CPU tests build
// them into a host program that runs the same arithmetic on recorded
// neighbourhoods and compares it with the FP64 oracle.
//
// Reference: src/meshoid/derivatives.py:27-138 builds, per particle, the basis
// a_j = [dx, dy, dz, dx^2/2, dy^2/2, dz^2/2, dx dy, dy dz, dz dx] of each
// neighbour's separation (scaled by 1/h here, so the matrix is O(1)), the
// kernel weights w_j = W(|dx_j| / h), L = sum_j w_j a_j a_j^T (:94-97) and
// R = w_j a_j (:99-101), and inverts L in FP64 (:132); D / D2 contract the
// weights with f_j - f_i (Meshoid.py:258,295).
//
// Why float-float: order-2 fits at 32 neighbours are sensitive.  Rounding the
// separations to FP32 (relative 6e-8) moves the FP64 answer by more than 1e-5
// on about a third of the rows of a clump mixture with fields that vary inside
// the kernel, so no method whose basis and weights carry FP32 precision meets
// 1e-5 there, whatever its solver.  Here the separations, the scaled
// coordinates, the weights, the basis, the moment matrix M and the right-hand
// sides b = sum_j w_j a_j (f_j - f_i) are float-float pairs (~2^-44
// relative), and M x = b is solved with a float-float Cholesky factor of M
// (backward stable; ~cond(M) * 1e-13 relative, against the ~6e-8 floor of an
// FP32 x that iterative refinement with an FP32 factor leaves, and which that
// refinement no longer reaches within a few steps past cond ~1e6).
#pragma once
#include "mg_chol.cuh"
#include "mg_ff.cuh"

namespace mg {

template <int DIM>
struct G2 {
    static constexpr int ND = DIM == 1 ? 2 : (DIM == 2 ? 5 : 9);
    static constexpr int NM = ND * (ND + 1) / 2;
};

__host__ __device__ __forceinline__ constexpr int g2_idx(int i, int j) {
    return i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i;
}

// Basis a and weighted basis w a of one neighbour from its separation d
// (float-float, unscaled) and 1/h (float-float).  Returns false when the
// neighbour lies outside the kernel (zero weight: it adds nothing).
template <int DIM>
__host__ __device__ __forceinline__ bool g2_basis(const ff d[3], ff hinv, bool weighted, ff a[G2<DIM>::ND],
                                                  ff wa[G2<DIM>::ND]) {
    constexpr int ND = G2<DIM>::ND;
    ff x[3], r2 = ff{0.0f, 0.0f};
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
        x[c] = ff_mul(d[c], hinv);
        r2 = ff_add(r2, ff_sqr(x[c]));
    }
    ff w = ff{1.0f, 0.0f};
    if (weighted) {
        w = ff_spline_w(ff_sqrt(r2), r2);
        if (w.hi == 0.0f) return false;
    }
#pragma unroll
    for (int m = 0; m < DIM; ++m) a[m] = x[m];
#pragma unroll
    for (int m = 0; m < DIM; ++m) {
        const ff s = ff_sqr(x[m]);
        a[DIM + m] = ff{0.5f * s.hi, 0.5f * s.lo};
    }
#pragma unroll
    for (int m = 0; m < ND - 2 * DIM; ++m) a[2 * DIM + m] = ff_mul(x[m % DIM], x[(m + 1) % DIM]);
#pragma unroll
    for (int m = 0; m < ND; ++m) wa[m] = ff_mul(w, a[m]);
    return true;
}

template <int DIM>
__host__ __device__ __forceinline__ void g2_moments_add(ff M[G2<DIM>::NM], const ff a[G2<DIM>::ND],
                                                        const ff wa[G2<DIM>::ND]) {
    constexpr int ND = G2<DIM>::ND;
#pragma unroll
    for (int i = 0; i < ND; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j) ff_fma_acc(M[i * (i + 1) / 2 + j], wa[i], a[j]);
}

template <int DIM>
__host__ __device__ __forceinline__ void g2_rhs_add(ff b[G2<DIM>::ND], const ff wa[G2<DIM>::ND], ff df) {
#pragma unroll
    for (int m = 0; m < G2<DIM>::ND; ++m) ff_fma_acc(b[m], wa[m], df);
}

// Float-float Cholesky factor of the packed moment matrix M = L L^T, in
// place: the strictly lower part becomes L, the diagonal 1 / L_jj (so that
// the solves multiply).  Backward stable like the FP64 factor, with the
// float-float unit (~2^-44) in place of FP64's: the solution of a row of
// condition c carries ~c * 1e-13 of itself.  Returns false when a pivot is
// not positive (the factor is then not usable).
template <int ND>
__host__ __device__ __forceinline__ bool g2_chol_ff(ff A[ND * (ND + 1) / 2]) {
    bool ok = true;
#pragma unroll
    for (int j = 0; j < ND; ++j) {
        ff s = A[g2_idx(j, j)];
#pragma unroll
        for (int p = 0; p < ND; ++p)
            if (p < j) ff_fma_acc(s, ff_neg(A[g2_idx(j, p)]), A[g2_idx(j, p)]);
        s = ff_norm(s);
        ok &= s.hi > 0.0f;
        if (!(s.hi > 0.0f)) s = ff{1.0f, 0.0f};
        const ff d = ff_sqrt(s);
        const ff r = ff_recip2(d.hi, d.lo);
        A[g2_idx(j, j)] = r;
#pragma unroll
        for (int i = 0; i < ND; ++i) {
            if (i <= j) continue;
            ff t = A[g2_idx(i, j)];
#pragma unroll
            for (int p = 0; p < ND; ++p)
                if (p < j) ff_fma_acc(t, ff_neg(A[g2_idx(i, p)]), A[g2_idx(j, p)]);
            A[g2_idx(i, j)] = ff_mul(ff_norm(t), r);
        }
    }
    return ok;
}

// x <- (L L^T)^-1 x with the factor of g2_chol_ff; lget(i) returns its packed
// entry i (float-float).
template <int ND, class LGet>
__host__ __device__ __forceinline__ void g2_solve_ff(LGet lget, ff x[ND]) {
#pragma unroll
    for (int i = 0; i < ND; ++i) {
        ff t = x[i];
#pragma unroll
        for (int p = 0; p < ND; ++p)
            if (p < i) ff_fma_acc(t, ff_neg(lget(g2_idx(i, p))), x[p]);
        x[i] = ff_mul(ff_norm(t), lget(g2_idx(i, i)));
    }
#pragma unroll
    for (int i = ND - 1; i >= 0; --i) {
        ff t = x[i];
#pragma unroll
        for (int p = 0; p < ND; ++p)
            if (p > i) ff_fma_acc(t, ff_neg(lget(g2_idx(p, i))), x[p]);
        x[i] = ff_mul(ff_norm(t), lget(g2_idx(i, i)));
    }
}

// FP64 solve of the order-2 system of one row from FP64 inputs (the
// reference's arithmetic, derivatives.py:27-138): the packed moment matrix is
// factored in place by FP64 Cholesky (pivots above 1e-14 of the largest
// diagonal entry).  A matrix that is not positive definite -- singular, where
// the reference raises LinAlgError (:132) or inverts a numerically singular
// matrix -- is factored again with a Tikhonov term 1e-12 of its largest
// diagonal entry added to the diagonal: its solution approaches the
// minimum-norm least-squares solution (the regularised directions have
// eigenvalues at most ~1e-14 of the largest, the others change by ~1e-12
// relative).  Returns true for such a row.
#ifdef __CUDA_ARCH__
#define MG_G2_NOINLINE __noinline__
#else
#define MG_G2_NOINLINE inline
#endif
template <int ND>
__host__ __device__ inline bool g2_chol64(double A[ND * (ND + 1) / 2], double shift, double tiny) {
    for (int j = 0; j < ND; ++j) {
        double s = A[g2_idx(j, j)] + shift;
        for (int p = 0; p < j; ++p) s -= A[g2_idx(j, p)] * A[g2_idx(j, p)];
        if (!(s > tiny)) return false;
        const double d = sqrt(s);
        A[g2_idx(j, j)] = d;
        const double inv = 1.0 / d;
        for (int i = j + 1; i < ND; ++i) {
            double t = A[g2_idx(i, j)];
            for (int p = 0; p < j; ++p) t -= A[g2_idx(i, p)] * A[g2_idx(j, p)];
            A[g2_idx(i, j)] = t * inv;
        }
    }
    return true;
}

template <int ND>
__host__ __device__ MG_G2_NOINLINE bool g2_factor64(double A[ND * (ND + 1) / 2]) {
    constexpr int NM = ND * (ND + 1) / 2;
    double amax = 0.0;
    for (int i = 0; i < ND; ++i) amax = fmax(amax, A[g2_idx(i, i)]);
    double B[NM];
    for (int i = 0; i < NM; ++i) B[i] = A[i];
    if (amax > 0.0 && g2_chol64<ND>(A, 0.0, 1e-14 * amax)) return false;
    for (int i = 0; i < NM; ++i) A[i] = B[i];
    const double lam = amax > 0.0 ? 1e-12 * amax : 1.0;
    if (!g2_chol64<ND>(A, lam, 0.0)) {
        // not even the shifted matrix factors (non-finite input): x = 0
        for (int i = 0; i < NM; ++i) A[i] = 0.0;
        for (int i = 0; i < ND; ++i) A[g2_idx(i, i)] = 1e300;
    }
    return true;
}

// x = A^-1 b with A the factor left by g2_factor64; b is overwritten by x.
template <int ND>
__host__ __device__ inline void g2_solve64(const double A[ND * (ND + 1) / 2], double b[ND]) {
#pragma unroll
    for (int i = 0; i < ND; ++i) {
        double t = b[i];
#pragma unroll
        for (int p = 0; p < ND; ++p)
            if (p < i) t -= A[i * (i + 1) / 2 + p] * b[p];
        b[i] = t / A[i * (i + 1) / 2 + i];
    }
#pragma unroll
    for (int ii = 0; ii < ND; ++ii) {
        const int i = ND - 1 - ii;
        double t = b[i];
#pragma unroll
        for (int p = 0; p < ND; ++p)
            if (p > i) t -= A[p * (p + 1) / 2 + i] * b[p];
        b[i] = t / A[i * (i + 1) / 2 + i];
    }
}

// FP64 basis of one neighbour from its FP64 separation d (unscaled) and 1/h;
// returns the weight (0 outside the kernel).
template <int DIM>
__host__ __device__ __forceinline__ double g2_basis64(const double d[3], double hinv, bool weighted,
                                                      double a[G2<DIM>::ND]) {
    constexpr int ND = G2<DIM>::ND;
    double x[3], r2 = 0.0;
    for (int c = 0; c < DIM; ++c) {
        x[c] = d[c] * hinv;
        r2 += x[c] * x[c];
    }
    double w = 1.0;
    if (weighted) {
        const double q = sqrt(r2);
        w = q <= 0.5 ? 1.0 - 6.0 * q * q + 6.0 * q * q * q : (q <= 1.0 ? 2.0 * (1.0 - q) * (1.0 - q) * (1.0 - q) : 0.0);
    }
    for (int m = 0; m < DIM; ++m) a[m] = x[m];
    for (int m = 0; m < DIM; ++m) a[DIM + m] = 0.5 * x[m] * x[m];
    for (int m = 0; m < ND - 2 * DIM; ++m) a[2 * DIM + m] = x[m % DIM] * x[(m + 1) % DIM];
    return w;
}

// Float-float root of norm * sum_j W(d_j / h) = k (HsmlIter's equation,
// src/meshoid/kernel_density.py:15-56) by STEPS Newton steps from an FP32
// root h0: n(h) - k in float-float from float-float distances, the slope in
// FP32 (from h0 ~1e-7 off, one step leaves ~1e-13).  dist(j) returns the
// j-th distance (float-float).  Returns h as hi + lo (normalised: hi is the
// FP32 rounding of the root); where a step would move h by more than 1e-4 (no
// isolated root nearby, e.g. coincident points) h0 is kept.
// KU > 0: k <= KU and the loop over the distances is unrolled KU times (the
// caller's row then stays in registers).
template <int DIM, int STEPS = 2, int KU = 0, class Dist>
__host__ __device__ __forceinline__ ff hsml_polish_ff(Dist dist, int k, float h0) {
    const ff norm = DIM == 3 ? ff_ratio(32.0f, 3.0f) : (DIM == 2 ? ff_ratio(40.0f, 7.0f) : ff_ratio(8.0f, 3.0f));
    ff h = ff{h0, 0.0f};
    for (int step = 0; step < STEPS; ++step) {
        const ff hinv = ff_recip2(h.hi, h.lo);
        ff s = ff{0.0f, 0.0f};
        float sdw = 0.0f;
        #pragma unroll
        for (int j = 0; j < (KU > 0 ? KU : k); ++j) {
            if (KU > 0 && j >= k) break;
            const ff q = ff_mul(dist(j), hinv);
            ff_acc(s, ff_spline_w(q, ff_sqr(q)));
            const float qf = q.hi;
            sdw += spline_dw(qf) * qf;
        }
        const ff n = ff_mul(norm, ff_norm(s));
        const float F = ff_to_f(ff_add_f(n, -(float)k));
        const float dF = -norm.hi * sdw * hinv.hi;  // dn/dh >= 0
        if (!(dF > 0.0f)) break;
        const float dh = -F / dF;
        if (!(fabsf(dh) <= 1e-4f * h.hi)) break;
        h = ff_add_f(h, dh);
    }
    return h;
}

}  // namespace mg
