// Kernel-weighted least-squares derivatives in one neighbour sweep, plus the
// kernel-weighted neighbour average and the field staging kernel.
//
// Reference: gradient_weights builds, per particle, the moment matrix
// L = sum_j w_j a_j a_j^T and R = w_j a_j (src/meshoid/derivatives.py:27-103),
// inverts L (:132) and caches L^-1 R (N, nd, k); D / D2 then contract the
// cached weights with f[ngb] - f[i] (src/meshoid/Meshoid.py:258,268,295).
// Here the contraction is folded into the sweep: each thread owns one query,
// accumulates L and the right-hand sides b_c = sum_j w_j a_j (f_c[j] - f_c[i])
// of every field component in registers, and solves L x = b_c at the end, so
// the (N, nd, k) weight tensor is never materialised.
//
// Precision: separations come from the FP32 hi/lo position split and field
// differences from the FP32 hi/lo field split, so every per-neighbour operand
// carries ~24 significant bits of the FP64 difference; coordinates are scaled
// by 1/h so L is O(1); sums are FP32; L is factored by FP32 Cholesky.  A
// non-positive pivot (singular / rank-deficient neighbourhood, where the
// reference raises LinAlgError) falls back to a Tikhonov-regularised solve
// and sets MG_Q_SINGULAR.
#include <atomic>

#include "mg_chol.cuh"
#include "mg_common.cuh"
#include "mg_ff.cuh"
#include "mg_refine.cuh"

namespace mg {

template <int DIM, int ORDER>
struct Basis {
    static constexpr int ND = ORDER == 1 ? DIM : (DIM == 1 ? 2 : (DIM == 2 ? 5 : 9));
    static constexpr int NM = ND * (ND + 1) / 2;
    // src/meshoid/derivatives.py:84-92 ordering: dx.., 0.5 dx^2.., cross terms
    __device__ __forceinline__ static void eval(const float x[3], float a[ND]) {
#pragma unroll
        for (int d = 0; d < DIM; ++d) a[d] = x[d];
        if (ORDER == 2) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) a[DIM + d] = 0.5f * x[d] * x[d];
#pragma unroll
            for (int d = 0; d < ND - 2 * DIM; ++d) a[2 * DIM + d] = x[d % DIM] * x[(d + 1) % DIM];
        }
    }
};

#ifndef MG_GRAD_UNROLL
#define MG_GRAD_UNROLL 4
#endif
constexpr int kGradUnroll = MG_GRAD_UNROLL;  // neighbours in flight per thread in k_grad
// MG_GRAD_MINB > 0: resident blocks of k_grad per SM its registers are cut
// for (0: the compiler's choice); MG_GRAD_NF8 0 caps an order-1 launch at 4
// components (more launches, fewer registers).
#ifndef MG_GRAD_MINB
#define MG_GRAD_MINB 0
#endif
#if MG_GRAD_MINB > 0
#define MG_GRAD_BOUNDS __launch_bounds__(128, MG_GRAD_MINB)
#else
#define MG_GRAD_BOUNDS __launch_bounds__(128)
#endif
#ifndef MG_GRAD_NF8
#define MG_GRAD_NF8 1
#endif
// FP32 rounding per term assumed by the order-1 sweep's error estimate,
// e ~ EB cond sum_j w |f_j - f_i| / |b| relative to x.  The estimate takes every
// rounding error aligned with the direction the matrix amplifies most; with
// half the unit roundoff (3e-8) the largest error over all rows stayed the
// same on the GPU (2^22 Plummer, 5 fields: 2.84e-6 with 0.49% of the rows
// re-solved in FP64, against 2.83e-6 with 1.79% at 6e-8; 2^22 clump
// mixture, 19 Fourier fields: 2.62e-6 with 0.26%, against 2.35e-6 with
// 0.61%; no row above 5e-6 in either), and the sweep took 0.36 ms less.
#ifndef MG_GRAD_EB
#define MG_GRAD_EB 3e-8f
#endif

struct GradArgs {
    int periodic;
    float box_hi, box_lo;
    const float4 *hi;
    const float4 *lo;
    const int32_t *queries;
    int64_t nq;
    const int32_t *ngb;
    int k;
    const float *hsml;
    const float *hsml_lo;  // may be NULL: h = hsml + hsml_lo (float-float)
    int weighted;
    const float *f_hi;
    const float *f_lo;
    int nf, nfp;   // components, row stride (multiple of 4)
    int c0;        // first component handled by this launch
    const int32_t *out_rows;
    float *d1;
    float *d2;
    int32_t *qstatus;
    // precise re-solve of ill-conditioned rows
    const double *pos64;
    double box;
    float cond_thr;
    int32_t *fix_queue;
    int32_t *fix_count;
    int32_t *fix_mark;  // per query: already queued (several component chunks may flag it)
    int refine;         // order 2: refine the FP32 answer once instead of queueing it (k_grad<..., true>)
};

// cholesky, chol_solve and cond_estimate: mg_chol.cuh

template <int DIM, int ORDER, int NF, bool REFINE = false>
__global__ MG_GRAD_BOUNDS void k_grad(GradArgs g) {
    static_assert(!REFINE || ORDER == 2, "the refinement step is for order 2");
    using B = Basis<DIM, ORDER>;
    constexpr int ND = B::ND, NM = B::NM;
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= g.nq) return;
    const int32_t p = g.queries ? g.queries[q] : (int32_t)q;
    const float4 h0 = g.hi[p], l0 = g.lo[p];
    // 1/h as a float-float pair: the scaling of every separation by 1/h is
    // coherent across the row, and least-squares fits can be sensitive to it
    // (1e-7 in h moved some rows' order-1 answers by 1e-5); the pair carries
    // it to ~2^-46, each scaled coordinate then rounds once on its own.
    const ff hv = ff_recip2(g.hsml[q], g.hsml_lo ? g.hsml_lo[q] : 0.0f);
    const float hinv = hv.hi, hinv_lo = hv.lo;

    float f0h[NF], f0l[NF];
    const float *rowh0 = g.f_hi + (int64_t)p * g.nfp + g.c0;
#pragma unroll
    for (int c = 0; c < NF; c += 4) {
        float4 v = *reinterpret_cast<const float4 *>(rowh0 + c);
        f0h[c] = v.x; f0h[c + 1] = v.y; f0h[c + 2] = v.z; f0h[c + 3] = v.w;
    }
    if (g.f_lo) {
        const float *rowl0 = g.f_lo + (int64_t)p * g.nfp + g.c0;
#pragma unroll
        for (int c = 0; c < NF; c += 4) {
            float4 v = *reinterpret_cast<const float4 *>(rowl0 + c);
            f0l[c] = v.x; f0l[c + 1] = v.y; f0l[c + 2] = v.z; f0l[c + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int c = 0; c < NF; ++c) f0l[c] = 0.0f;
    }

    // Right-hand sides are summed with Kahan compensation: a field that varies
    // on the kernel scale makes |b| much smaller than its terms, and plain FP32
    // summation error (~sqrt(k) 6e-8 of the terms) would then dominate.
    float M[NM];
    float rhs[NF][ND], rcmp[NF][ND];
    float cabs[NF];  // sum_j w |f_j - f_i|: bounds the terms of each right-hand side
#pragma unroll
    for (int i = 0; i < NM; ++i) M[i] = 0.0f;
#pragma unroll
    for (int c = 0; c < NF; ++c) {
        cabs[c] = 0.0f;
#pragma unroll
        for (int m = 0; m < ND; ++m) rhs[c][m] = rcmp[c][m] = 0.0f;
    }

    const int32_t *nb = g.ngb + q * g.k;
    // unrolled so the gathers of several neighbours are in flight together;
    // a zero weight contributes nothing, so no branch is needed
#pragma unroll kGradUnroll
    for (int j = 0; j < g.k; ++j) {
        const int32_t s = __ldg(nb + j);
        const float4 hb = __ldg(g.hi + s), lb = __ldg(g.lo + s);
        float3 d = g.periodic ? sep_hilo_periodic(h0, l0, hb, lb, g.box_hi, g.box_lo)
                              : sep_hilo(h0, l0, hb, lb);
        const float x[3] = {scale_sep(d.x, hinv, hinv_lo), scale_sep(d.y, hinv, hinv_lo),
                            scale_sep(d.z, hinv, hinv_lo)};
        float r2 = 0.0f;
#pragma unroll
        for (int a = 0; a < DIM; ++a) r2 += x[a] * x[a];
        const float w = g.weighted ? spline_w(sqrtf(r2)) : 1.0f;
        float a[ND], wa[ND];
        B::eval(x, a);
#pragma unroll
        for (int m = 0; m < ND; ++m) wa[m] = w * a[m];
#pragma unroll
        for (int i = 0; i < ND; ++i)
#pragma unroll
            for (int jj = 0; jj <= i; ++jj) M[i * (i + 1) / 2 + jj] += wa[i] * a[jj];
        const float *rh = g.f_hi + (int64_t)s * g.nfp + g.c0;
        const float *rl = g.f_lo ? g.f_lo + (int64_t)s * g.nfp + g.c0 : nullptr;
#pragma unroll
        for (int c = 0; c < NF; c += 4) {
            const float4 vh = __ldg(reinterpret_cast<const float4 *>(rh + c));
            float4 vl = make_float4(0.f, 0.f, 0.f, 0.f);
            if (rl) vl = __ldg(reinterpret_cast<const float4 *>(rl + c));
            const float df[4] = {(vh.x - f0h[c]) + (vl.x - f0l[c]), (vh.y - f0h[c + 1]) + (vl.y - f0l[c + 1]),
                                 (vh.z - f0h[c + 2]) + (vl.z - f0l[c + 2]),
                                 (vh.w - f0h[c + 3]) + (vl.w - f0l[c + 3])};
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                cabs[c + u] += w * fabsf(df[u]);
#pragma unroll
                for (int m = 0; m < ND; ++m) {
                    const float y = __fmaf_rn(wa[m], df[u], -rcmp[c + u][m]);
                    const float t = __fadd_rn(rhs[c + u][m], y);
                    rcmp[c + u][m] = __fsub_rn(__fsub_rn(t, rhs[c + u][m]), y);
                    rhs[c + u][m] = t;
                }
            }
        }
    }

    // Factor L.  A failed factorisation, or a condition number above cond_thr
    // (FP32 normal equations lose ~cond * 6e-8 relative accuracy), queues the
    // row for the FP64 re-solve in k_grad_fix, which overwrites this result.
    // So does a solution whose estimated FP32 error exceeds the derivative
    // tolerance (1e-5, plus 2e-6 cond at order 2) relative to its
    // first-derivative part or, at order 2, to its second-derivative part
    // (small against the first-derivative part for a smooth field, which the
    // matrix rounding, ~6e-8 cond ||x||, reaches first); and one whose
    // right-hand side cancels so strongly that the rounding of its terms,
    // ~6e-8 cond sum_j w |f_j - f_i| / |b|, does.
    float L[NM];
#pragma unroll
    for (int i = 0; i < NM; ++i) L[i] = M[i];
    bool flag = false;
    float cond = 1.0f;
    if (!cholesky<ND>(L)) {
#pragma unroll
        for (int i = 0; i < NM; ++i) L[i] = 0.0f;
#pragma unroll
        for (int i = 0; i < ND; ++i) L[i * (i + 1) / 2 + i] = 1e30f;
        flag = true;
    } else {
        cond = cond_estimate<ND>(M, L);
        flag = cond > g.cond_thr;
    }
    {
        // the hi/lo positions' representation error, ~1.2e-14 |x| of each
        // separation (|x| frame-relative, or the box side), against h: order
        // 1 (cond <= 30 unflagged) above 1e-7 / cond of h, order 2 above 1e-9
        // of h, the row is re-solved from the FP64 positions
        float xq = fmaxf(fabsf(h0.x), fmaxf(fabsf(h0.y), fabsf(h0.z)));
        if (g.periodic) xq = fmaxf(xq, g.box_hi);
        const float rep = 1.2e-14f * xq * hinv;
        flag |= ORDER == 1 ? rep * cond > 1e-7f : rep > 1e-9f;
    }
    const float tol = 1e-5f + (ORDER == 2 ? 2e-6f * cond : 0.0f);
    const int ncomp = min(NF, g.nf - g.c0);
    const float h2inv = hinv * hinv;
    const int64_t orow = g.out_rows ? (int64_t)g.out_rows[q] : q;
    if constexpr (!REFINE) {
#pragma unroll
        for (int c = 0; c < NF; ++c) {
            // a guard, not a break: with no exit from the unrolled loop every
            // index stays constant
            if (c < ncomp) {
            float x[ND];
#pragma unroll
            for (int m = 0; m < ND; ++m) x[m] = rhs[c][m];
            chol_solve<ND>(L, x);
            {
                float n1 = 0.0f, n2 = 0.0f, nb = 0.0f;
#pragma unroll
                for (int m = 0; m < ND; ++m) {
                    (m < DIM ? n1 : n2) += x[m] * x[m];
                    nb += rhs[c][m] * rhs[c][m];
                }
                // matrix rounding, relative to ||x|| (order 2: the unit
                // roundoff, as in the refinement branch below)
                const float em = (ORDER == 1 ? MG_GRAD_EB : 6e-8f) * cond;
                if (ORDER == 2) flag |= em * em * (n1 + n2) > tol * tol * n2;
                const float eb = em * cabs[c];  // right-hand-side rounding, relative to |b|
                flag |= eb * eb > tol * tol * nb;
            }
            float *o1 = g.d1 + (orow * g.nf + g.c0 + c) * DIM;
#pragma unroll
            for (int m = 0; m < DIM; ++m) o1[m] = x[m] * hinv;
            if (ORDER == 2 && g.d2) {
                float *o2 = g.d2 + (orow * g.nf + g.c0 + c) * (ND - DIM);
#pragma unroll
                for (int m = DIM; m < ND; ++m) o2[m - DIM] = x[m] * h2inv;
            }
            }
        }
    } else {
        // Order 2 with one refinement step in place of most FP64 re-solves.
        // The matrix rounding error of the FP32 answer, ~6e-8 cond ||x||, is
        // spread over all its parts; against the second-derivative part, much
        // smaller than the first-derivative part for a smooth field, it often
        // exceeds the tolerance.  Its source is the FP32 rounding of the
        // separations in the moment matrix and the right-hand side.  One step
        // x += (L L^T)^-1 r, r = sum_j w_j a_j e_j with the residual
        // e_j = (f_j - f_i) - a_j . x evaluated with the field difference and
        // the linear part of the prediction as float-float pairs (hi/lo
        // splits, TwoSum, the FMA error of each product), removes it: the
        // first-derivative part of the prediction cancels exactly, and the
        // remaining error is ~6e-8 cond ||correction||.  Rows whose factor
        // failed or whose condition estimate exceeds cond_thr, and rows whose
        // right-hand side cancels too strongly, still go to the FP64 re-solve.
        const float em = 6e-8f * cond;
        bool need = false;
#pragma unroll
        for (int c = 0; c < NF; ++c) {
            if (c >= ncomp) break;
            float n1 = 0.0f, n2 = 0.0f, nbb = 0.0f;
#pragma unroll
            for (int m = 0; m < ND; ++m) nbb += rhs[c][m] * rhs[c][m];
            chol_solve<ND>(L, rhs[c]);  // rhs[c] holds the solution from here on
#pragma unroll
            for (int m = 0; m < ND; ++m) (m < DIM ? n1 : n2) += rhs[c][m] * rhs[c][m];
            need |= em * em * (n1 + n2) > tol * tol * n2;
            const float eb = em * cabs[c];
            flag |= eb * eb > tol * tol * nbb;
        }
        if (need && !flag) {
            float (&res)[NF][ND] = rcmp;  // the compensation terms are no longer needed
#pragma unroll
            for (int c = 0; c < NF; ++c)
#pragma unroll
                for (int m = 0; m < ND; ++m) res[c][m] = 0.0f;
#pragma unroll kGradUnroll
            for (int j = 0; j < g.k; ++j) {
                const int32_t s = __ldg(nb + j);
                const float4 hb = __ldg(g.hi + s), lb = __ldg(g.lo + s);
                float dv[3], dl[3];
                if (g.periodic) {
                    dv[0] = wrap1_ff(hb.x, h0.x, lb.x, l0.x, g.box_hi, g.box_lo, dl[0]);
                    dv[1] = wrap1_ff(hb.y, h0.y, lb.y, l0.y, g.box_hi, g.box_lo, dl[1]);
                    dv[2] = wrap1_ff(hb.z, h0.z, lb.z, l0.z, g.box_hi, g.box_lo, dl[2]);
                } else {
                    dv[0] = sep1_ff(hb.x, h0.x, lb.x, l0.x, dl[0]);
                    dv[1] = sep1_ff(hb.y, h0.y, lb.y, l0.y, dl[1]);
                    dv[2] = sep1_ff(hb.z, h0.z, lb.z, l0.z, dl[2]);
                }
                const float x[3] = {scale_sep(dv[0], hinv, hinv_lo), scale_sep(dv[1], hinv, hinv_lo),
                                    scale_sep(dv[2], hinv, hinv_lo)};
                float r2 = 0.0f;
#pragma unroll
                for (int a = 0; a < DIM; ++a) r2 += x[a] * x[a];
                const float w = g.weighted ? spline_w(sqrtf(r2)) : 1.0f;
                float a[ND], wa[ND], xl[3];
                B::eval(x, a);
#pragma unroll
                for (int m = 0; m < ND; ++m) wa[m] = w * a[m];
#pragma unroll
                for (int d = 0; d < DIM; ++d) xl[d] = scaled_sep_lo2(dv[d], dl[d], hinv, hinv_lo, x[d]);
                const float *rh = g.f_hi + (int64_t)s * g.nfp + g.c0;
                const float *rl = g.f_lo ? g.f_lo + (int64_t)s * g.nfp + g.c0 : nullptr;
#pragma unroll
                for (int c = 0; c < NF; c += 4) {
                    const float4 vh = __ldg(reinterpret_cast<const float4 *>(rh + c));
                    float4 vl = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (rl) vl = __ldg(reinterpret_cast<const float4 *>(rl + c));
                    const float fh[4] = {vh.x, vh.y, vh.z, vh.w}, fl[4] = {vl.x, vl.y, vl.z, vl.w};
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int cc = c + u;
                        const float e =
                            refine_residual<DIM, ND>(x, xl, a, rhs[cc], fh[u], fl[u], f0h[cc], f0l[cc]);
#pragma unroll
                        for (int m = 0; m < ND; ++m) res[cc][m] = fmaf(wa[m], e, res[cc][m]);
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < NF; ++c) {
                if (c >= ncomp) break;
                chol_solve<ND>(L, res[c]);
                float dn = 0.0f, n2 = 0.0f;
#pragma unroll
                for (int m = 0; m < ND; ++m) {
                    rhs[c][m] += res[c][m];
                    dn += res[c][m] * res[c][m];
                    if (m >= DIM) n2 += rhs[c][m] * rhs[c][m];
                }
                // the refined answer's error, ~6e-8 cond ||correction||
                flag |= em * em * dn > tol * tol * n2;
            }
            // a row that still fails goes on to the FP64 re-solve and is not
            // marked refined (k_grad_fix also clears the mark that an earlier
            // component chunk of the row may have set)
            if (g.qstatus && !flag) atomicOr(g.qstatus + q, MG_Q_REFINED);
        } else if (need) {
            flag = true;
        }
#pragma unroll
        for (int c = 0; c < NF; ++c) {
            if (c >= ncomp) break;
            float *o1 = g.d1 + (orow * g.nf + g.c0 + c) * DIM;
#pragma unroll
            for (int m = 0; m < DIM; ++m) o1[m] = rhs[c][m] * hinv;
            if (g.d2) {
                float *o2 = g.d2 + (orow * g.nf + g.c0 + c) * (ND - DIM);
#pragma unroll
                for (int m = DIM; m < ND; ++m) o2[m - DIM] = rhs[c][m] * h2inv;
            }
        }
    }
    if (flag && g.fix_queue && atomicExch(g.fix_mark + q, 1) == 0) {
        const int slot = atomicAdd(g.fix_count, 1);
        g.fix_queue[slot] = (int32_t)q;
    }
}

// ---- FP64 re-solve of queued (ill-conditioned or singular) rows ------------------
// Follows the reference arithmetic: FP64 separations from the FP64 positions,
// FP64 kernel weights and moment sums (src/meshoid/derivatives.py:27-103).
// The moment matrix (scaled by h) is solved by FP64 Cholesky; when that fails
// (rank-deficient neighbourhood -- the reference raises LinAlgError here) the
// minimum-norm solution from a Jacobi eigen-decomposition (pseudo-inverse,
// eigenvalues below 1e-12 of the largest dropped) is used and MG_Q_SINGULAR
// is set.
template <int ND>
__device__ void jacobi_pinv(double A[ND][ND], double P[ND][ND]) {
    double V[ND][ND];
    for (int i = 0; i < ND; ++i)
        for (int j = 0; j < ND; ++j) V[i][j] = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 30; ++sweep) {
        double off = 0.0;
        for (int i = 0; i < ND; ++i)
            for (int j = i + 1; j < ND; ++j) off += A[i][j] * A[i][j];
        if (off < 1e-30) break;
        for (int p = 0; p < ND; ++p)
            for (int q = p + 1; q < ND; ++q) {
                if (fabs(A[p][q]) < 1e-300) continue;
                const double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < ND; ++k) {
                    const double akp = A[k][p], akq = A[k][q];
                    A[k][p] = c * akp - sn * akq;
                    A[k][q] = sn * akp + c * akq;
                }
                for (int k = 0; k < ND; ++k) {
                    const double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = c * apk - sn * aqk;
                    A[q][k] = sn * apk + c * aqk;
                }
                for (int k = 0; k < ND; ++k) {
                    const double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - sn * vkq;
                    V[k][q] = sn * vkp + c * vkq;
                }
            }
    }
    double emax = 0.0;
    for (int i = 0; i < ND; ++i) emax = fmax(emax, fabs(A[i][i]));
    for (int i = 0; i < ND; ++i)
        for (int j = 0; j < ND; ++j) {
            double acc = 0.0;
            for (int k = 0; k < ND; ++k) {
                const double e = A[k][k];
                if (fabs(e) > 1e-12 * emax) acc += V[i][k] * V[j][k] / e;
            }
            P[i][j] = acc;
        }
}

template <int DIM, int ORDER>
__global__ __launch_bounds__(128) void k_grad_fix(GradArgs g) {
    using B = Basis<DIM, ORDER>;
    constexpr int ND = B::ND;
    const int nfix = *g.fix_count;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nfix; e += gridDim.x * blockDim.x) {
        const int64_t q = g.fix_queue[e];
        const int32_t p = g.queries ? g.queries[q] : (int32_t)q;
        const double h = (double)g.hsml[q] + (g.hsml_lo ? (double)g.hsml_lo[q] : 0.0), hinv = 1.0 / h;
        const int32_t *nb = g.ngb + q * g.k;
        double A[ND][ND];
        for (int i = 0; i < ND; ++i)
            for (int j = 0; j < ND; ++j) A[i][j] = 0.0;
        auto basis = [&](int32_t s, double a[ND]) -> double {
            double x[3] = {0.0, 0.0, 0.0}, r2 = 0.0;
            for (int c = 0; c < DIM; ++c) {
                double d = g.pos64[(int64_t)s * 3 + c] - g.pos64[(int64_t)p * 3 + c];
                if (g.periodic && fabs(d) > 0.5 * g.box) d = -copysign(g.box - fabs(d), d);
                x[c] = d * hinv;
                r2 += x[c] * x[c];
            }
            const double qq = sqrt(r2);
            double w = 1.0;
            if (g.weighted) w = qq <= 0.5 ? 1.0 - 6.0 * qq * qq + 6.0 * qq * qq * qq
                                          : (qq <= 1.0 ? 2.0 * (1.0 - qq) * (1.0 - qq) * (1.0 - qq) : 0.0);
            for (int d = 0; d < DIM; ++d) a[d] = x[d];
            if (ORDER == 2) {
                for (int d = 0; d < DIM; ++d) a[DIM + d] = 0.5 * x[d] * x[d];
                for (int d = 0; d < ND - 2 * DIM; ++d) a[2 * DIM + d] = x[d % DIM] * x[(d + 1) % DIM];
            }
            return w;
        };
        auto fval = [&](int32_t s, int c) -> double {
            return (double)g.f_hi[(int64_t)s * g.nfp + c] + (g.f_lo ? (double)g.f_lo[(int64_t)s * g.nfp + c] : 0.0);
        };
        const int64_t orow = g.out_rows ? (int64_t)g.out_rows[q] : q;
        if (g.qstatus) {
            atomicOr(g.qstatus + q, MG_Q_FP64_SOLVE);
            atomicAnd(g.qstatus + q, ~MG_Q_REFINED);
        }
        // Right-hand sides G components at a time, one basis evaluation per
        // neighbour and group; the moment matrix is summed in the first group's
        // pass (FP64 runs at a small fraction of the FP32 rate on this GPU, so
        // the basis is not recomputed for it).
        constexpr int G = ORDER == 1 ? 8 : 4;
        double P[ND][ND];
        for (int c0 = 0; c0 < g.nf; c0 += G) {
            const int nc = min(G, g.nf - c0);
            double f0[G], b[G][ND];
            for (int u = 0; u < G; ++u) {
                f0[u] = u < nc ? fval(p, c0 + u) : 0.0;
                for (int i = 0; i < ND; ++i) b[u][i] = 0.0;
            }
            for (int j = 0; j < g.k; ++j) {
                const int32_t s = nb[j];
                double a[ND];
                const double w = basis(s, a);
                if (w == 0.0) continue;
                if (c0 == 0) {
                    for (int i = 0; i < ND; ++i) {
                        const double wa = w * a[i];
                        for (int jj = 0; jj <= i; ++jj) A[i][jj] += wa * a[jj];
                    }
                }
                for (int u = 0; u < G; ++u) {
                    if (u >= nc) break;
                    const double df = fval(s, c0 + u) - f0[u];
                    for (int i = 0; i < ND; ++i) b[u][i] += w * a[i] * df;
                }
            }
            if (c0 == 0) {
                for (int i = 0; i < ND; ++i)
                    for (int jj = i + 1; jj < ND; ++jj) A[i][jj] = A[jj][i];
                // inverse (Cholesky-based when SPD, pseudo-inverse otherwise)
                bool spd = true;
                double Lc[ND][ND];
                for (int i = 0; i < ND; ++i)
                    for (int j = 0; j < ND; ++j) Lc[i][j] = 0.0;
                for (int j = 0; j < ND && spd; ++j) {
                    double sdiag = A[j][j];
                    for (int k2 = 0; k2 < j; ++k2) sdiag -= Lc[j][k2] * Lc[j][k2];
                    if (!(sdiag > 1e-14 * fmax(A[0][0], 1e-300))) {
                        spd = false;
                        break;
                    }
                    Lc[j][j] = sqrt(sdiag);
                    for (int i = j + 1; i < ND; ++i) {
                        double t = A[i][j];
                        for (int k2 = 0; k2 < j; ++k2) t -= Lc[i][k2] * Lc[j][k2];
                        Lc[i][j] = t / Lc[j][j];
                    }
                }
                if (spd) {
                    for (int c = 0; c < ND; ++c) {
                        double x[ND];
                        for (int i = 0; i < ND; ++i) {
                            double t = (i == c) ? 1.0 : 0.0;
                            for (int k2 = 0; k2 < i; ++k2) t -= Lc[i][k2] * x[k2];
                            x[i] = t / Lc[i][i];
                        }
                        for (int i = ND - 1; i >= 0; --i) {
                            double t = x[i];
                            for (int k2 = i + 1; k2 < ND; ++k2) t -= Lc[k2][i] * x[k2];
                            x[i] = t / Lc[i][i];
                        }
                        for (int i = 0; i < ND; ++i) P[i][c] = x[i];
                    }
                } else {
                    double Ac[ND][ND];
                    for (int i = 0; i < ND; ++i)
                        for (int j = 0; j < ND; ++j) Ac[i][j] = A[i][j];
                    jacobi_pinv<ND>(Ac, P);
                    if (g.qstatus) atomicOr(g.qstatus + q, MG_Q_SINGULAR);
                }
            }
            for (int u = 0; u < nc; ++u) {
                double x[ND];
                for (int i = 0; i < ND; ++i) {
                    double t = 0.0;
                    for (int j = 0; j < ND; ++j) t += P[i][j] * b[u][j];
                    x[i] = t;
                }
                const int c = c0 + u;
                float *o1 = g.d1 + (orow * g.nf + c) * DIM;
                for (int m = 0; m < DIM; ++m) o1[m] = (float)(x[m] * hinv);
                if (ORDER == 2 && g.d2) {
                    float *o2 = g.d2 + (orow * g.nf + c) * (ND - DIM);
                    for (int m = DIM; m < ND; ++m) o2[m - DIM] = (float)(x[m] * hinv * hinv);
                }
            }
        }
    }
}

template <int DIM, int ORDER>
static int launch_grad(const GradArgs &g0, cudaStream_t st) {
    GradArgs g = g0;
    const unsigned blocks = (unsigned)((g.nq + 127) / 128);
    // Components per launch: up to 8 (order 1) or 4 (order 2), as many as the
    // registers hold with the compensated sums.  A launch with NF components
    // reads columns [c0, c0 + NF) of rows of stride nfp, so NF never exceeds
    // nfp - c0 (both multiples of 4).
    for (int c0 = 0; c0 < g.nfp;) {
        g.c0 = c0;
        const int rem = g.nfp - c0;
        int nf_launch = 4;
        if constexpr (ORDER == 1) {
            if (MG_GRAD_NF8 && rem >= 8) {
                k_grad<DIM, ORDER, 8><<<blocks, 128, 0, st>>>(g);
                nf_launch = 8;
            } else {
                k_grad<DIM, ORDER, 4><<<blocks, 128, 0, st>>>(g);
            }
        } else if (g.refine) {
            k_grad<DIM, ORDER, 4, true><<<blocks, 128, 0, st>>>(g);
        } else {
            k_grad<DIM, ORDER, 4><<<blocks, 128, 0, st>>>(g);
        }
        MG_CHECK_LAUNCH();
        c0 += nf_launch;
    }
    if (g.fix_queue) {
        int dev = 0, nsm = 148;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        const int64_t want = (g.nq + 127) / 128;
        const unsigned fb = (unsigned)(want < (int64_t)nsm * 4 ? want : (int64_t)nsm * 4);
        k_grad_fix<DIM, ORDER><<<fb, 128, 0, st>>>(g);
        MG_CHECK_LAUNCH();
    }
    return MG_OK;
}

// ---- kernel-weighted average -----------------------------------------------------
__global__ __launch_bounds__(128) void k_kernel_average(GradArgs g, double *__restrict__ out) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= g.nq) return;
    const int32_t p = g.queries ? g.queries[q] : (int32_t)q;
    const float4 h0 = g.hi[p], l0 = g.lo[p];
    const float hinv = 1.0f / g.hsml[q];
    const int32_t *nb = g.ngb + q * g.k;
    float wsum = 0.0f;
    for (int j = 0; j < g.k; ++j) {
        const int32_t s = __ldg(nb + j);
        float3 d = g.periodic ? sep_hilo_periodic(h0, l0, __ldg(g.hi + s), __ldg(g.lo + s), g.box_hi, g.box_lo)
                              : sep_hilo(h0, l0, __ldg(g.hi + s), __ldg(g.lo + s));
        wsum += spline_w(sqrtf(d.x * d.x + d.y * d.y + d.z * d.z) * hinv);
    }
    const float winv = 1.0f / wsum;
    for (int c = 0; c < g.nf; ++c) {
        double acc = 0.0;
        float accf = 0.0f, comp = 0.0f;
        for (int j = 0; j < g.k; ++j) {
            const int32_t s = __ldg(nb + j);
            float3 d = g.periodic ? sep_hilo_periodic(h0, l0, __ldg(g.hi + s), __ldg(g.lo + s), g.box_hi, g.box_lo)
                                  : sep_hilo(h0, l0, __ldg(g.hi + s), __ldg(g.lo + s));
            const float w = spline_w(sqrtf(d.x * d.x + d.y * d.y + d.z * d.z) * hinv) * winv;
            const float fv = g.f_hi[(int64_t)s * g.nfp + c];
            const float fl = g.f_lo ? g.f_lo[(int64_t)s * g.nfp + c] : 0.0f;
            // compensated sum of w * (hi + lo)
            float y = fmaf(w, fv, -comp) + w * fl;
            float t = accf + y;
            comp = (t - accf) - y;
            accf = t;
        }
        acc = (double)accf - (double)comp;
        out[(g.out_rows ? (int64_t)g.out_rows[q] : q) * g.nf + c] = acc;
    }
}

// ---- standard deviation over the neighbours -----------------------------------------
// np.std(f[ngb], axis=1) of src/meshoid/Meshoid.py:351-366: population standard
// deviation of each component over the k neighbours (self included), two
// passes in FP64 on the hi + lo values.
__global__ __launch_bounds__(128) void k_kernel_variance(GradArgs g, double *__restrict__ out) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= g.nq) return;
    const int32_t *nb = g.ngb + q * g.k;
    const double kinv = 1.0 / (double)g.k;
    auto fval = [&](int32_t s, int c) -> double {
        return (double)g.f_hi[(int64_t)s * g.nfp + c] + (g.f_lo ? (double)g.f_lo[(int64_t)s * g.nfp + c] : 0.0);
    };
    for (int c = 0; c < g.nf; ++c) {
        double mean = 0.0;
        for (int j = 0; j < g.k; ++j) mean += fval(__ldg(nb + j), c);
        mean *= kinv;
        double ss = 0.0;
        for (int j = 0; j < g.k; ++j) {
            const double d = fval(__ldg(nb + j), c) - mean;
            ss += d * d;
        }
        out[(g.out_rows ? (int64_t)g.out_rows[q] : q) * g.nf + c] = sqrt(ss * kinv);
    }
}

// ---- field staging: particle order FP64 -> slot order FP32 hi/lo -------------------
__global__ void k_load_fields(const double *__restrict__ f, const int32_t *__restrict__ order,
                              int64_t n, int nf, int nfp, float *__restrict__ hi,
                              float *__restrict__ lo) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= n * nfp) return;
    const int64_t s = idx / nfp;
    const int c = (int)(idx - s * nfp);
    double v = 0.0;
    if (c < nf) v = f[(int64_t)order[s] * nf + c];
    const float h = (float)v;
    hi[idx] = h;
    if (lo) lo[idx] = (float)(v - (double)h);
}

}  // namespace mg

using namespace mg;

// Process-wide switch of the order-2 refinement step (k_grad<..., true>);
// off by default.  Atomic so that one host thread may flip it while another
// launches sweeps.
static std::atomic<int> g_grad_refine{0};

extern "C" int mg_grad_set_refine(int32_t enabled) {
    return g_grad_refine.exchange(enabled ? 1 : 0);
}

static inline void grad_common(GradArgs &g, const mg_cells *c) {
    g.periodic = c->boxsize > 0;
    g.box_hi = (float)c->boxsize;
    g.box_lo = (float)(c->boxsize - (double)g.box_hi);
    g.hi = reinterpret_cast<const float4 *>(c->pos_hi);
    g.lo = reinterpret_cast<const float4 *>(c->pos_lo);
}

extern "C" int mg_load_fields(const mg_cells *c, const double *f, int32_t nf, float *hi, float *lo,
                              void *stream_) {
    if (!c || !f || !hi || nf < 1) return MG_ERR_ARG;
    const int nfp = (nf + 3) & ~3;
    const int64_t tot = c->n * nfp;
    k_load_fields<<<(unsigned)((tot + 255) / 256), 256, 0, as_stream(stream_)>>>(f, c->order, c->n, nf, nfp,
                                                                                 hi, lo);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" size_t mg_grad_sweep_workspace_bytes(int64_t nq) {
    return nq > 0 ? 2 * align_up(sizeof(int32_t) * nq) + 512 : 0;
}

extern "C" int mg_grad_sweep(const mg_cells *c, const int32_t *queries, int64_t nq, const int32_t *ngb,
                             int32_t k, const float *hsml, const float *hsml_lo, int32_t order, int32_t weighted,
                             const float *f_hi, const float *f_lo, int32_t nf, const int32_t *out_rows,
                             float *d1, float *d2, int32_t *qstatus, float cond_threshold, void *workspace,
                             size_t workspace_bytes, void *stream_) {
    if (!c || nq <= 0 || !ngb || !hsml || !f_hi || !d1 || nf < 1) return MG_ERR_ARG;
    if (workspace && workspace_bytes < mg_grad_sweep_workspace_bytes(nq)) return MG_ERR_ARG;
    if (order != 1 && order != 2) return MG_ERR_ARG;
    if (order == 2 && !d2) return MG_ERR_ARG;
    if (k < 1 || k > MG_MAX_K) return MG_ERR_UNSUPPORTED;
    GradArgs g{};
    grad_common(g, c);
    g.queries = queries;
    g.nq = nq;
    g.ngb = ngb;
    g.k = k;
    g.hsml = hsml;
    g.hsml_lo = hsml_lo;
    g.weighted = weighted;
    g.f_hi = f_hi;
    g.f_lo = f_lo;
    g.nf = nf;
    g.nfp = (nf + 3) & ~3;
    g.c0 = 0;
    g.out_rows = out_rows;
    g.d1 = d1;
    g.d2 = d2;
    g.qstatus = qstatus;
    g.pos64 = c->pos64;
    g.box = c->boxsize;
    g.cond_thr = cond_threshold > 0.0f ? cond_threshold : 3.0e38f;
    g.fix_queue = nullptr;
    g.fix_count = nullptr;
    g.fix_mark = nullptr;
    g.refine = order == 2 && g_grad_refine.load() ? 1 : 0;
    cudaStream_t st = as_stream(stream_);
    if (workspace) {
        Carve w(workspace, workspace_bytes);
        g.fix_queue = w.take<int32_t>(nq);
        g.fix_mark = w.take<int32_t>(nq);
        g.fix_count = w.take<int32_t>(4);
        if (!w.ok()) return MG_ERR_ARG;
        MG_CUDA(cudaMemsetAsync(g.fix_count, 0, sizeof(int32_t), st));
        MG_CUDA(cudaMemsetAsync(g.fix_mark, 0, sizeof(int32_t) * nq, st));
    }
    const int dim = c->dim;
    if (order == 1) {
        if (dim == 1) return launch_grad<1, 1>(g, st);
        if (dim == 2) return launch_grad<2, 1>(g, st);
        return launch_grad<3, 1>(g, st);
    }
    if (dim == 1) return launch_grad<1, 2>(g, st);
    if (dim == 2) return launch_grad<2, 2>(g, st);
    return launch_grad<3, 2>(g, st);
}

extern "C" int mg_kernel_average(const mg_cells *c, const int32_t *queries, int64_t nq, const int32_t *ngb,
                                 int32_t k, const float *hsml, const float *f_hi, const float *f_lo,
                                 int32_t nf, const int32_t *out_rows, double *out, void *stream_) {
    if (!c || nq <= 0 || !ngb || !hsml || !f_hi || !out || nf < 1) return MG_ERR_ARG;
    GradArgs g{};
    grad_common(g, c);
    g.queries = queries;
    g.nq = nq;
    g.ngb = ngb;
    g.k = k;
    g.hsml = hsml;
    g.f_hi = f_hi;
    g.f_lo = f_lo;
    g.nf = nf;
    g.nfp = (nf + 3) & ~3;
    g.out_rows = out_rows;
    k_kernel_average<<<(unsigned)((nq + 127) / 128), 128, 0, as_stream(stream_)>>>(g, out);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" int mg_kernel_variance(const mg_cells *c, const int32_t *queries, int64_t nq, const int32_t *ngb,
                                  int32_t k, const float *f_hi, const float *f_lo, int32_t nf, const int32_t *out_rows,
                                  double *out, void *stream_) {
    if (!c || nq <= 0 || !ngb || !f_hi || !out || nf < 1 || k < 1) return MG_ERR_ARG;
    GradArgs g{};
    grad_common(g, c);
    g.queries = queries;
    g.nq = nq;
    g.ngb = ngb;
    g.k = k;
    g.f_hi = f_hi;
    g.f_lo = f_lo;
    g.nf = nf;
    g.nfp = (nf + 3) & ~3;
    g.out_rows = out_rows;
    k_kernel_variance<<<(unsigned)((nq + 127) / 128), 128, 0, as_stream(stream_)>>>(g, out);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

// ---- gradient sweep without allocation --------------------------------------------
// Some callers cannot allocate device memory at the point where they need
// derivatives: a simulation or visualisation code that reserves its whole GPU
// memory budget for its own pool at start-up, or a tight per-step loop whose
// owner forbids allocator calls (they may synchronise the device or fail once
// the pool is exhausted).  mg_grad_sweep_noalloc serves them: it is
// mg_grad_sweep with its scratch (the queue of rows re-solved in FP64 and their
// marks) taken
// from a fixed array compiled into this library instead of a caller workspace.
//
// Limit: nq <= MG_NOALLOC_MAX_QUERIES.  The array (about 16 MiB) is resident on
// every GPU that loads the library, until the process exits.  Every call
// shares it, so calls that overlap on the GPU race on it: a call's results
// depend on the array until its last kernel (the FP64 re-solve) has finished,
// so order whole calls on the GPU -- one stream, or a wait on an event
// recorded after the previous call -- not only on the host.  The queue
// counter and the marks are cleared at the start of each call; the queue
// keeps whatever the last call left.
// Each call looks up the array's device address on the current device
// (cudaGetSymbolAddress, which allocates nothing), so the address is never
// stale after a device reset; on a device's first call that lookup also loads
// the library's module there, so make that first call before any stream
// capture.
static __device__ __align__(256) int32_t g_noalloc_scratch[2 * MG_NOALLOC_MAX_QUERIES + 256];

static int32_t *noalloc_scratch_for_current_device(int &status) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
        status = MG_ERR_CUDA;
        return nullptr;
    }
    status = MG_OK;
    return static_cast<int32_t *>(p);
}

extern "C" int mg_grad_sweep_noalloc(const mg_cells *c, const int32_t *queries, int64_t nq, const int32_t *ngb,
                                     int32_t k, const float *hsml, const float *hsml_lo, int32_t order,
                                     int32_t weighted,
                                     const float *f_hi, const float *f_lo, int32_t nf, const int32_t *out_rows,
                                     float *d1, float *d2, int32_t *qstatus, float cond_threshold,
                                     void *stream_) {
    if (nq > MG_NOALLOC_MAX_QUERIES) return MG_ERR_NOALLOC_LIMIT;
    int status = MG_OK;
    int32_t *scratch = noalloc_scratch_for_current_device(status);
    if (!scratch) return status;
    static_assert(sizeof(g_noalloc_scratch) >=
                      2 * ((MG_NOALLOC_MAX_QUERIES * sizeof(int32_t) + 255) / 256 * 256) + 512,
                  "fixed scratch must hold the largest workspace mg_grad_sweep asks for");
    return mg_grad_sweep(c, queries, nq, ngb, k, hsml, hsml_lo, order, weighted, f_hi, f_lo, nf, out_rows, d1, d2,
                         qstatus,
                         cond_threshold, scratch, sizeof(g_noalloc_scratch), stream_);
}
