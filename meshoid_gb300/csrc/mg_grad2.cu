// Order-2 least-squares derivatives (D order 2, D2) in float-float, with the
// float-float smoothing-length polish they are evaluated at and the
// three-plane field split they read.
//
// Reference: src/meshoid/derivatives.py:27-138 (weights), Meshoid.py:110-140
// (ComputeDWeights caches them), :237-295 (D / D2 contract them with
// f[ngb] - f[i]).  The weights cache has an analogue here: the per-row
// float-float moment matrices ("moments", mg_grad2_moments), computed once per
// neighbour set and reused by every mg_grad2_solve call; rows that need the
// FP64 path are listed in a queue kept with them.
//
// Passes:
//   k_g2_moments   thread per query: float-float M over the k neighbours,
//                  FP32 Cholesky + condition estimate, then the float-float
//                  Cholesky factor of M, which is what is cached.  Rows that
//                  are singular or above the condition threshold are queued
//                  for the FP64 re-solve (the queue is part of the cache).
//   k_g2_rhs       thread per query and chunk of NF components: float-float
//                  right-hand sides over the neighbours, then a float-float
//                  solve with the cached factor per component.  Rows queued by
//                  the moments pass are skipped; a row whose solution is not
//                  finite is queued for the FP64 re-solve of this call.
//   k_g2_fix64     thread per queued row: the reference's arithmetic in FP64
//                  from the FP64 positions and fields (moment matrix,
//                  right-hand sides of every component, Cholesky or, when
//                  singular, a Tikhonov-regularised Cholesky).
#include "mg_common.cuh"
#include "mg_grad2.cuh"
#include "mg_refine.cuh"

namespace mg {

constexpr int kG2NF = 4;       // components per rhs launch
constexpr int kG2FixG = 4;     // components per right-hand-side pass of the FP64 re-solve
#ifndef MG_G2_RHS_MINB
#define MG_G2_RHS_MINB 2  // resident blocks of k_g2_rhs per SM the registers are cut for
#endif

struct G2Args {
    int periodic;
    float box_hi, box_lo;
    const float4 *hi;
    const float4 *lo;
    const int32_t *queries;
    int64_t nq;
    const int32_t *ngb;
    int k;
    const float *hsml;
    const float *hsml_lo;
    int weighted;
    float cond_thr;
    float2 *mom;       // [NM][nq] float-float Cholesky factor of each row's moment matrix
    int32_t *mflag;    // [nq] 1: the row is solved in FP64 (queued by the moments pass)
    int32_t *queue;    // rows queued by the moments pass
    int32_t *qcount;
    const double *pos64;
    double box;
    const float *f_hi, *f_mid, *f_lo;
    int nf, nfp, c0;
    const int32_t *out_rows;
    float *d1, *d2;
    int32_t *qstatus;
    int32_t *mark;     // [nq] row queued by the rhs pass
    int32_t *queue2;
    int32_t *q2count;
};

__device__ __forceinline__ void g2_sep(const G2Args &g, float4 h0, float4 l0, int32_t s, ff d[3]) {
    const float4 hb = __ldg(g.hi + s), lb = __ldg(g.lo + s);
    float lo;
    if (g.periodic) {
        d[0].hi = wrap1_ff(hb.x, h0.x, lb.x, l0.x, g.box_hi, g.box_lo, lo); d[0].lo = lo;
        d[1].hi = wrap1_ff(hb.y, h0.y, lb.y, l0.y, g.box_hi, g.box_lo, lo); d[1].lo = lo;
        d[2].hi = wrap1_ff(hb.z, h0.z, lb.z, l0.z, g.box_hi, g.box_lo, lo); d[2].lo = lo;
    } else {
        d[0].hi = sep1_ff(hb.x, h0.x, lb.x, l0.x, lo); d[0].lo = lo;
        d[1].hi = sep1_ff(hb.y, h0.y, lb.y, l0.y, lo); d[1].lo = lo;
        d[2].hi = sep1_ff(hb.z, h0.z, lb.z, l0.z, lo); d[2].lo = lo;
    }
}

__device__ __forceinline__ ff g2_hinv(const G2Args &g, int64_t q) {
    return ff_recip2(g.hsml[q], g.hsml_lo ? g.hsml_lo[q] : 0.0f);
}

template <int DIM>
__global__ __launch_bounds__(128) void k_g2_moments(const __grid_constant__ G2Args g) {
    constexpr int ND = G2<DIM>::ND, NM = G2<DIM>::NM;
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= g.nq) return;
    const int32_t p = g.queries ? g.queries[q] : (int32_t)q;
    const float4 h0 = g.hi[p], l0 = g.lo[p];
    const ff hinv = g2_hinv(g, q);
    ff M[NM];
#pragma unroll
    for (int i = 0; i < NM; ++i) M[i] = ff{0.0f, 0.0f};
    const int32_t *nb = g.ngb + q * g.k;
    for (int j = 0; j < g.k; ++j) {
        ff d[3], a[ND], wa[ND];
        g2_sep(g, h0, l0, __ldg(nb + j), d);
        if (g2_basis<DIM>(d, hinv, g.weighted, a, wa)) g2_moments_add<DIM>(M, a, wa);
    }
    float Mh[NM], L[NM];
#pragma unroll
    for (int i = 0; i < NM; ++i) {
        M[i] = ff_norm(M[i]);
        Mh[i] = L[i] = M[i].hi;
    }
    bool flag = !cholesky_nb<ND>(L);
    if (!flag) {
        const float cond = cond_estimate<ND>(Mh, L);
        flag = !(cond <= g.cond_thr);
        // the hi/lo positions' representation error, ~1.2e-14 |x| of each
        // separation, against h: above 1e-9 of h (a clump ~1e-5 of its
        // distance from the frame centre across; the densest clumps of the
        // 2^24 clump mixture are at ~3e-10) FP64 positions instead
        float xq = fmaxf(fabsf(h0.x), fmaxf(fabsf(h0.y), fabsf(h0.z)));
        if (g.periodic) xq = fmaxf(xq, g.box_hi);
        flag |= 1.2e-14f * xq * hinv.hi > 1e-9f;
    }
    flag |= !g2_chol_ff<ND>(M);
#pragma unroll
    for (int i = 0; i < NM; ++i) g.mom[(int64_t)i * g.nq + q] = make_float2(M[i].hi, M[i].lo);
    g.mflag[q] = flag ? 1 : 0;
    if (flag) g.queue[atomicAdd(g.qcount, 1)] = (int32_t)q;
}

template <int DIM, int NF>
__global__ __launch_bounds__(128, MG_G2_RHS_MINB) void k_g2_rhs(const __grid_constant__ G2Args g) {
    constexpr int ND = G2<DIM>::ND, NM = G2<DIM>::NM;
    __shared__ float2 sb[NF * ND * 128];  // [component * ND + m][thread]: normalised right-hand sides
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.nq;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = e;
        if (g.mflag[q]) continue;  // solved in FP64 by k_g2_fix64
        const int32_t p = g.queries ? g.queries[q] : (int32_t)q;
        const float4 h0 = g.hi[p], l0 = g.lo[p];
        const ff hinv = g2_hinv(g, q);
        float f0h[NF], f0m[NF], f0l[NF];
        const int64_t r0 = (int64_t)p * g.nfp + g.c0;
#pragma unroll
        for (int c = 0; c < NF; c += 4) {
            const float4 vh = *reinterpret_cast<const float4 *>(g.f_hi + r0 + c);
            const float4 vm = *reinterpret_cast<const float4 *>(g.f_mid + r0 + c);
            const float4 vl = *reinterpret_cast<const float4 *>(g.f_lo + r0 + c);
            f0h[c] = vh.x; f0h[c + 1] = vh.y; f0h[c + 2] = vh.z; f0h[c + 3] = vh.w;
            f0m[c] = vm.x; f0m[c + 1] = vm.y; f0m[c + 2] = vm.z; f0m[c + 3] = vm.w;
            f0l[c] = vl.x; f0l[c + 1] = vl.y; f0l[c + 2] = vl.z; f0l[c + 3] = vl.w;
        }
        ff b[NF][ND];
#pragma unroll
        for (int c = 0; c < NF; ++c)
#pragma unroll
            for (int m = 0; m < ND; ++m) b[c][m] = ff{0.0f, 0.0f};
        const int32_t *nb = g.ngb + q * g.k;
        for (int j = 0; j < g.k; ++j) {
            const int32_t s = __ldg(nb + j);
            ff d[3], a[ND], wa[ND];
            g2_sep(g, h0, l0, s, d);
            if (!g2_basis<DIM>(d, hinv, g.weighted, a, wa)) continue;
            const int64_t rs = (int64_t)s * g.nfp + g.c0;
#pragma unroll
            for (int c = 0; c < NF; c += 4) {
                const float4 vh = __ldg(reinterpret_cast<const float4 *>(g.f_hi + rs + c));
                const float4 vm = __ldg(reinterpret_cast<const float4 *>(g.f_mid + rs + c));
                const float4 vl = __ldg(reinterpret_cast<const float4 *>(g.f_lo + rs + c));
                const float fh[4] = {vh.x, vh.y, vh.z, vh.w}, fm[4] = {vm.x, vm.y, vm.z, vm.w},
                            fl[4] = {vl.x, vl.y, vl.z, vl.w};
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    g2_rhs_add<DIM>(b[c + u], wa, ff_diff3(fh[u], fm[u], fl[u], f0h[c + u], f0m[c + u], f0l[c + u]));
            }
        }
        const int ncomp = min(NF, g.nf - g.c0);
        const int64_t orow = g.out_rows ? (int64_t)g.out_rows[q] : q;
        const float hi1 = hinv.hi, hi2 = hinv.hi * hinv.hi;
        // The right-hand sides wait in shared memory (this thread's column)
        // while the components are solved one after another by a single copy
        // of the solve: unrolled over the components, the kernel outgrew the
        // instruction cache and stalled on instruction fetch.
#pragma unroll
        for (int c = 0; c < NF; ++c)
#pragma unroll
            for (int m = 0; m < ND; ++m) {
                const ff v = ff_norm(b[c][m]);
                sb[(c * ND + m) * 128 + threadIdx.x] = make_float2(v.hi, v.lo);
            }
        ff L[NM];  // the float-float Cholesky factor of the moments pass
#pragma unroll
        for (int i = 0; i < NM; ++i) {
            const float2 v = g.mom[(int64_t)i * g.nq + q];
            L[i] = ff{v.x, v.y};
        }
        bool ok = true;
#pragma unroll 1
        for (int c = 0; c < ncomp; ++c) {
            ff x[ND];
#pragma unroll
            for (int m = 0; m < ND; ++m) {
                const float2 v = sb[(c * ND + m) * 128 + threadIdx.x];
                x[m] = ff{v.x, v.y};
            }
            g2_solve_ff<ND>([&](int i) { return L[i]; }, x);
            float *o1 = g.d1 + (orow * g.nf + g.c0 + c) * DIM;
#pragma unroll
            for (int m = 0; m < DIM; ++m) {
                o1[m] = x[m].hi * hi1;
                ok &= isfinite(x[m].hi);
            }
            if (g.d2) {
                float *o2 = g.d2 + (orow * g.nf + g.c0 + c) * (ND - DIM);
#pragma unroll
                for (int m = DIM; m < ND; ++m) o2[m - DIM] = x[m].hi * hi2;
            }
#pragma unroll
            for (int m = DIM; m < ND; ++m) ok &= isfinite(x[m].hi);
        }
        if (!ok && atomicExch(g.mark + q, 1) == 0) g.queue2[atomicAdd(g.q2count, 1)] = (int32_t)q;
    }
}

// The reference's arithmetic in FP64 for the queued rows (derivatives.py:
// 27-138): FP64 separations from the FP64 positions, FP64 weights and basis,
// the moment matrix factored once (Cholesky, regularised when singular), right-hand sides of kG2FixG components per pass over the
// neighbours; fields as the FP64 sum of their three planes, h as hi + lo.
template <int DIM>
__global__ __launch_bounds__(64) void k_g2_fix64(const __grid_constant__ G2Args g, const int32_t *__restrict__ queue,
                                                 const int32_t *__restrict__ count) {
    constexpr int ND = G2<DIM>::ND, NM = G2<DIM>::NM, G = kG2FixG;
    const int n = *count;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int64_t q = queue[e];
        const int32_t p = g.queries ? g.queries[q] : (int32_t)q;
        double h = (double)g.hsml[q] + (g.hsml_lo ? (double)g.hsml_lo[q] : 0.0);
        double p0[3] = {0.0, 0.0, 0.0};
        for (int c = 0; c < DIM; ++c) p0[c] = g.pos64[(int64_t)p * 3 + c];
        const int32_t *nb = g.ngb + q * g.k;
        auto sep64 = [&](int32_t s, double d[3]) {
            d[0] = d[1] = d[2] = 0.0;
            for (int c = 0; c < DIM; ++c) {
                double t = g.pos64[(int64_t)s * 3 + c] - p0[c];
                if (g.periodic && fabs(t) > 0.5 * g.box) t = -copysign(g.box - fabs(t), t);
                d[c] = t;
            }
        };
        // These rows are the sensitive ones: h to FP64 precision as well, by
        // two Newton steps on HsmlIter's equation (kernel_density.py:15-56)
        // from the FP64 distances (the float-float h carries the 2^-48
        // relative precision of the hi/lo positions).
        if (g.weighted) {
            const double norm = DIM == 3 ? 32.0 / 3.0 : (DIM == 2 ? 40.0 / 7.0 : 8.0 / 3.0);
            for (int it = 0; it < 2; ++it) {
                double n = 0.0, sdw = 0.0;
                const double hi_ = 1.0 / h;
                for (int j = 0; j < g.k; ++j) {
                    double d[3];
                    sep64(nb[j], d);
                    const double qq = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) * hi_;
                    n += qq <= 0.5 ? 1.0 - 6.0 * qq * qq + 6.0 * qq * qq * qq
                                   : (qq <= 1.0 ? 2.0 * (1.0 - qq) * (1.0 - qq) * (1.0 - qq) : 0.0);
                    sdw += (qq <= 0.5 ? qq * (18.0 * qq - 12.0) : (qq <= 1.0 ? -6.0 * (1.0 - qq) * (1.0 - qq) : 0.0)) * qq;
                }
                const double F = norm * n - (double)g.k, dF = -norm * sdw * hi_;
                if (!(dF > 0.0)) break;
                const double step = -F / dF;
                if (!(fabs(step) <= 1e-6 * h)) break;
                h += step;
            }
        }
        const double hinv = 1.0 / h;
        auto fval = [&](int32_t s, int c) -> double {
            const int64_t i = (int64_t)s * g.nfp + c;
            return ((double)g.f_hi[i] + (double)g.f_mid[i]) + (double)g.f_lo[i];
        };
        const int64_t orow = g.out_rows ? (int64_t)g.out_rows[q] : q;
        double A[NM];
        for (int i = 0; i < NM; ++i) A[i] = 0.0;
        bool pinv = false;
        for (int c0 = 0; c0 < g.nf; c0 += G) {
            const int nc = min(G, g.nf - c0);
            double f0[G], b[G][ND];
#pragma unroll
            for (int u = 0; u < G; ++u) {
                f0[u] = u < nc ? fval(p, c0 + u) : 0.0;
#pragma unroll
                for (int m = 0; m < ND; ++m) b[u][m] = 0.0;
            }
            for (int j = 0; j < g.k; ++j) {
                const int32_t s = nb[j];
                double d[3], a[ND];
                sep64(s, d);
                const double w = g2_basis64<DIM>(d, hinv, g.weighted, a);
                if (w == 0.0) continue;
                if (c0 == 0) {
#pragma unroll
                    for (int i = 0; i < ND; ++i) {
                        const double wai = w * a[i];
#pragma unroll
                        for (int jj = 0; jj < ND; ++jj)
                            if (jj <= i) A[i * (i + 1) / 2 + jj] += wai * a[jj];
                    }
                }
#pragma unroll
                for (int u = 0; u < G; ++u) {
                    if (u < nc) {
                        const double wdf = w * (fval(s, c0 + u) - f0[u]);
#pragma unroll
                        for (int m = 0; m < ND; ++m) b[u][m] += wdf * a[m];
                    }
                }
            }
            if (c0 == 0) {
                double Af[NM];  // factored out of line (the regularised retry keeps a copy)
#pragma unroll
                for (int i = 0; i < NM; ++i) Af[i] = A[i];
                pinv = g2_factor64<ND>(Af);
#pragma unroll
                for (int i = 0; i < NM; ++i) A[i] = Af[i];
            }
#pragma unroll
            for (int u = 0; u < G; ++u) {
                if (u >= nc) break;
                g2_solve64<ND>(A, b[u]);
                float *o1 = g.d1 + (orow * g.nf + c0 + u) * DIM;
                for (int m = 0; m < DIM; ++m) o1[m] = (float)(b[u][m] * hinv);
                if (g.d2) {
                    float *o2 = g.d2 + (orow * g.nf + c0 + u) * (ND - DIM);
                    for (int m = DIM; m < ND; ++m) o2[m - DIM] = (float)(b[u][m] * hinv * hinv);
                }
            }
        }
        if (g.qstatus) atomicOr(g.qstatus + q, MG_Q_FP64_SOLVE | (pinv ? MG_Q_SINGULAR : 0));
    }
}

// Float-float smoothing lengths from the neighbour rows (HsmlIter's root,
// kernel_density.py:15-56): two Newton steps from the FP32 solve.
template <int DIM>
__global__ __launch_bounds__(128) void k_hsml_polish(const __grid_constant__ G2Args g, float *__restrict__ h_hi,
                                                     float *__restrict__ h_lo) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= g.nq) return;
    const int32_t p = g.queries ? g.queries[q] : (int32_t)q;
    const float4 h0 = g.hi[p], l0 = g.lo[p];
    const int32_t *nb = g.ngb + q * g.k;
    auto dist = [&](int j) -> ff {
        ff d[3];
        g2_sep(g, h0, l0, __ldg(nb + j), d);
        ff r2 = ff{0.0f, 0.0f};
#pragma unroll
        for (int c = 0; c < DIM; ++c) r2 = ff_add(r2, ff_sqr(d[c]));
        return ff_sqrt(r2);
    };
    const ff h = hsml_polish_ff<DIM>(dist, g.k, g.hsml[q]);
    h_hi[q] = h.hi;
    h_lo[q] = h.lo;
}

// f (particle order, FP64) -> slot order three-plane split hi + mid + lo
__global__ void k_load_fields3(const double *__restrict__ f, const int32_t *__restrict__ order, int64_t n, int nf,
                               int nfp, float *__restrict__ hi, float *__restrict__ mid, float *__restrict__ lo) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= n * nfp) return;
    const int64_t s = idx / nfp;
    const int c = (int)(idx - s * nfp);
    double v = 0.0;
    if (c < nf) v = f[(int64_t)order[s] * nf + c];
    const float h = (float)v;
    const double r = v - (double)h;
    const float m = (float)r;
    hi[idx] = h;
    mid[idx] = m;
    lo[idx] = (float)(r - (double)m);
}

}  // namespace mg

using namespace mg;

static inline void g2_common(G2Args &g, const mg_cells *c, const int32_t *queries, int64_t nq, const int32_t *ngb,
                             int32_t k, const float *hsml, const float *hsml_lo, int32_t weighted) {
    g = G2Args{};
    g.periodic = c->boxsize > 0;
    g.pos64 = c->pos64;
    g.box = c->boxsize;
    g.box_hi = (float)c->boxsize;
    g.box_lo = (float)(c->boxsize - (double)g.box_hi);
    g.hi = reinterpret_cast<const float4 *>(c->pos_hi);
    g.lo = reinterpret_cast<const float4 *>(c->pos_lo);
    g.queries = queries;
    g.nq = nq;
    g.ngb = ngb;
    g.k = k;
    g.hsml = hsml;
    g.hsml_lo = hsml_lo;
    g.weighted = weighted;
}

static inline int g2_nm(int dim) { return dim == 1 ? 3 : (dim == 2 ? 15 : 45); }

extern "C" size_t mg_grad2_moments_bytes(int64_t nq, int32_t dim) {
    if (nq <= 0 || dim < 1 || dim > 3) return 0;
    return align_up(sizeof(float2) * (size_t)g2_nm(dim) * nq) + align_up(sizeof(int32_t) * nq) +
           align_up(sizeof(int32_t) * nq) + 512;
}

namespace {
struct MomView {
    float2 *mom;
    int32_t *mflag, *queue, *qcount;
};
bool carve_moments(void *buf, size_t bytes, int64_t nq, int dim, MomView &v) {
    Carve w(buf, bytes);
    v.mom = w.take<float2>((size_t)g2_nm(dim) * nq);
    v.mflag = w.take<int32_t>(nq);
    v.queue = w.take<int32_t>(nq);
    v.qcount = w.take<int32_t>(4);
    return w.ok();
}
int nsm_count() {
    int dev = 0, nsm = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    return nsm;
}
}  // namespace

template <int DIM>
static int launch_moments(G2Args g, cudaStream_t st) {
    k_g2_moments<DIM><<<(unsigned)((g.nq + 127) / 128), 128, 0, st>>>(g);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" int mg_grad2_moments(const mg_cells *c, const int32_t *queries, int64_t nq, const int32_t *ngb,
                                int32_t k, const float *hsml, const float *hsml_lo, int32_t weighted,
                                float cond_threshold, void *moments, size_t moments_bytes, void *stream_) {
    if (!c || nq <= 0 || !ngb || !hsml || !moments || k < 1 || k > MG_MAX_K) return MG_ERR_ARG;
    if (c->dim < 1 || c->dim > 3 || moments_bytes < mg_grad2_moments_bytes(nq, c->dim)) return MG_ERR_ARG;
    G2Args g;
    g2_common(g, c, queries, nq, ngb, k, hsml, hsml_lo, weighted);
    MomView v;
    if (!carve_moments(moments, moments_bytes, nq, c->dim, v)) return MG_ERR_ARG;
    g.mom = v.mom;
    g.mflag = v.mflag;
    g.queue = v.queue;
    g.qcount = v.qcount;
    g.cond_thr = cond_threshold > 0.0f ? cond_threshold : 3.0e38f;
    cudaStream_t st = as_stream(stream_);
    MG_CUDA(cudaMemsetAsync(v.qcount, 0, sizeof(int32_t), st));
    if (c->dim == 1) return launch_moments<1>(g, st);
    if (c->dim == 2) return launch_moments<2>(g, st);
    return launch_moments<3>(g, st);
}

extern "C" size_t mg_grad2_solve_workspace_bytes(int64_t nq) {
    return nq > 0 ? 2 * align_up(sizeof(int32_t) * nq) + 512 : 0;
}

template <int DIM>
static int launch_rhs(G2Args g, cudaStream_t st) {
    for (int c0 = 0; c0 < g.nf; c0 += kG2NF) {
        g.c0 = c0;
        k_g2_rhs<DIM, kG2NF><<<(unsigned)((g.nq + 127) / 128), 128, 0, st>>>(g);
        MG_CHECK_LAUNCH();
    }
    // rows queued by the moments pass, then rows whose solution was not finite
    const unsigned persist = (unsigned)nsm_count() * 8;
    k_g2_fix64<DIM><<<persist, 64, 0, st>>>(g, g.queue, g.qcount);
    MG_CHECK_LAUNCH();
    k_g2_fix64<DIM><<<persist, 64, 0, st>>>(g, g.queue2, g.q2count);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" int mg_grad2_solve(const mg_cells *c, const int32_t *queries, int64_t nq, const int32_t *ngb, int32_t k,
                              const float *hsml, const float *hsml_lo, int32_t weighted, void *moments,
                              size_t moments_bytes, const float *f_hi, const float *f_mid, const float *f_lo,
                              int32_t nf, const int32_t *out_rows, float *d1, float *d2, int32_t *qstatus,
                              void *workspace, size_t workspace_bytes, void *stream_) {
    if (!c || nq <= 0 || !ngb || !hsml || !moments || !f_hi || !f_mid || !f_lo || !d1 || nf < 1) return MG_ERR_ARG;
    if (k < 1 || k > MG_MAX_K || c->dim < 1 || c->dim > 3) return MG_ERR_ARG;
    if (moments_bytes < mg_grad2_moments_bytes(nq, c->dim)) return MG_ERR_ARG;
    if (!workspace || workspace_bytes < mg_grad2_solve_workspace_bytes(nq)) return MG_ERR_ARG;
    G2Args g;
    g2_common(g, c, queries, nq, ngb, k, hsml, hsml_lo, weighted);
    MomView v;
    if (!carve_moments(moments, moments_bytes, nq, c->dim, v)) return MG_ERR_ARG;
    g.mom = v.mom;
    g.mflag = v.mflag;
    g.queue = v.queue;
    g.qcount = v.qcount;
    g.f_hi = f_hi;
    g.f_mid = f_mid;
    g.f_lo = f_lo;
    g.nf = nf;
    g.nfp = (nf + 3) & ~3;
    g.out_rows = out_rows;
    g.d1 = d1;
    g.d2 = d2;
    g.qstatus = qstatus;
    Carve w(workspace, workspace_bytes);
    g.mark = w.take<int32_t>(nq);
    g.queue2 = w.take<int32_t>(nq);
    g.q2count = w.take<int32_t>(4);
    if (!w.ok()) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    MG_CUDA(cudaMemsetAsync(g.q2count, 0, sizeof(int32_t), st));
    MG_CUDA(cudaMemsetAsync(g.mark, 0, sizeof(int32_t) * nq, st));
    if (c->dim == 1) return launch_rhs<1>(g, st);
    if (c->dim == 2) return launch_rhs<2>(g, st);
    return launch_rhs<3>(g, st);
}

extern "C" int mg_hsml_polish(const mg_cells *c, const int32_t *queries, int64_t nq, const int32_t *ngb, int32_t k,
                              const float *hsml, float *hsml_hi, float *hsml_lo, void *stream_) {
    if (!c || nq <= 0 || !ngb || !hsml || !hsml_hi || !hsml_lo || k < 1 || k > MG_MAX_K) return MG_ERR_ARG;
    G2Args g;
    g2_common(g, c, queries, nq, ngb, k, hsml, nullptr, 1);
    cudaStream_t st = as_stream(stream_);
    const unsigned blocks = (unsigned)((nq + 127) / 128);
    if (c->dim == 1)
        k_hsml_polish<1><<<blocks, 128, 0, st>>>(g, hsml_hi, hsml_lo);
    else if (c->dim == 2)
        k_hsml_polish<2><<<blocks, 128, 0, st>>>(g, hsml_hi, hsml_lo);
    else
        k_hsml_polish<3><<<blocks, 128, 0, st>>>(g, hsml_hi, hsml_lo);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" int mg_load_fields3(const mg_cells *c, const double *f, int32_t nf, float *hi, float *mid, float *lo,
                               void *stream_) {
    if (!c || !f || !hi || !mid || !lo || nf < 1) return MG_ERR_ARG;
    const int nfp = (nf + 3) & ~3;
    const int64_t tot = c->n * nfp;
    k_load_fields3<<<(unsigned)((tot + 255) / 256), 256, 0, as_stream(stream_)>>>(f, c->order, c->n, nf, nfp, hi, mid,
                                                                                  lo);
    MG_CHECK_LAUNCH();
    return MG_OK;
}
