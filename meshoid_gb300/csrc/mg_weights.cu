// Explicit weight matrices and the 1-D KDE of the reference's Meshoid:
//   mg_kernel_weights    get_kernel_weights   src/meshoid/Meshoid.py:172-177
//   mg_gradient_weights  gradient_weights     src/meshoid/derivatives.py:27-138
//                        (ComputeDWeights      src/meshoid/Meshoid.py:110-140)
//   mg_kde_1d            KDE                  src/meshoid/Meshoid.py:722-750
//
// The derivatives themselves never need the (N, nd, k) weights (the gradient
// sweep contracts on the fly); these entry points materialise them for
// callers that read them.  FP64 throughout, as the reference computes them.
#include "mg_common.cuh"

namespace mg {

// src/meshoid/kernel_density.py:82-96 (Kernel), FP64
__device__ __forceinline__ double kernel64(double q) {
    if (q <= 0.5) return 1.0 - 6.0 * q * q + 6.0 * q * q * q;
    if (q <= 1.0) {
        const double a = 1.0 - q;
        return 2.0 * a * a * a;
    }
    return 0.0;
}

__global__ void k_kernel_weights(const double *__restrict__ ngbdist, const double *__restrict__ h, int64_t nq, int k,
                                 double *__restrict__ w) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const double hinv = 1.0 / h[q];
    double s = 0.0;
    for (int j = 0; j < k; ++j) s += kernel64(ngbdist[q * k + j] * hinv);
    for (int j = 0; j < k; ++j) w[q * k + j] = kernel64(ngbdist[q * k + j] * hinv) / s;
}

// Basis of derivatives.py:84-92: dx..., 0.5 dx^2..., dx_d dx_{(d+1) % dim}.
template <int DIM, int ORDER>
struct Basis64 {
    static constexpr int ND = ORDER == 1 ? DIM : (DIM == 1 ? 2 : (DIM == 2 ? 5 : 9));
    __device__ __forceinline__ static void eval(const double x[3], double a[ND]) {
#pragma unroll
        for (int d = 0; d < DIM; ++d) a[d] = x[d];
        if (ORDER == 2) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) a[DIM + d] = 0.5 * x[d] * x[d];
#pragma unroll
            for (int d = 0; d < ND - 2 * DIM; ++d) a[2 * DIM + d] = x[d % DIM] * x[(d + 1) % DIM];
        }
    }
};

__device__ __forceinline__ double nearest_image64(double d, double box) {
    if (box > 0.0 && fabs(d) > box / 2) return -copysign(box - fabs(d), d);
    return d;
}

// One thread per query: dx and kernel weights of its neighbours, the normal
// matrix L = sum w a a^T, its inverse by Gauss-Jordan with partial pivoting,
// then W = L^-1 (w a) column by column.  An exactly singular L (no usable
// pivot) leaves the row NaN and is counted: the reference raises
// LinAlgError there (derivatives.py:132).
template <int DIM, int ORDER>
__global__ __launch_bounds__(128) void k_gradient_weights(const double *__restrict__ pos,
                                                         const int64_t *__restrict__ ngb, int k,
                                                         const double *__restrict__ h,
                                                         const int64_t *__restrict__ indices, int64_t nq, double box,
                                                         bool weighted, double *__restrict__ out,
                                                         unsigned long long *__restrict__ n_singular) {
    using B = Basis64<DIM, ORDER>;
    constexpr int ND = B::ND;
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int64_t i = indices[q];
    const double hinv = 1.0 / h[q];
    double L[ND][ND], inv[ND][ND];
#pragma unroll
    for (int a = 0; a < ND; ++a)
#pragma unroll
        for (int b = 0; b < ND; ++b) {
            L[a][b] = 0.0;
            inv[a][b] = a == b ? 1.0 : 0.0;
        }
    auto neighbour = [&](int j, double av[ND], double &w) {
        const int64_t n = ngb[q * k + j];
        double x[3] = {0.0, 0.0, 0.0}, r = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            x[d] = nearest_image64(pos[n * DIM + d] - pos[i * DIM + d], box);
            r += x[d] * x[d];
        }
        w = weighted ? kernel64(sqrt(r) * hinv) : 1.0;
        B::eval(x, av);
    };
    for (int j = 0; j < k; ++j) {
        double av[ND], w;
        neighbour(j, av, w);
#pragma unroll
        for (int a = 0; a < ND; ++a)
#pragma unroll
            for (int b = 0; b < ND; ++b) L[a][b] += av[a] * av[b] * w;
    }
    bool singular = false;
    // rolled: the pivot rows are run-time indices (the arrays live in local memory)
#pragma unroll 1
    for (int c = 0; c < ND; ++c) {
        int piv = c;
        double best = fabs(L[c][c]);
#pragma unroll 1
        for (int r = c + 1; r < ND; ++r)
            if (fabs(L[r][c]) > best) {
                best = fabs(L[r][c]);
                piv = r;
            }
        if (best == 0.0) {
            singular = true;
            break;
        }
        if (piv != c) {
#pragma unroll
            for (int b = 0; b < ND; ++b) {
                const double t = L[c][b];
                L[c][b] = L[piv][b];
                L[piv][b] = t;
                const double u = inv[c][b];
                inv[c][b] = inv[piv][b];
                inv[piv][b] = u;
            }
        }
        const double pinv = 1.0 / L[c][c];
#pragma unroll
        for (int b = 0; b < ND; ++b) {
            L[c][b] *= pinv;
            inv[c][b] *= pinv;
        }
#pragma unroll 1
        for (int r = 0; r < ND; ++r) {
            if (r == c) continue;
            const double fct = L[r][c];
#pragma unroll
            for (int b = 0; b < ND; ++b) {
                L[r][b] -= fct * L[c][b];
                inv[r][b] -= fct * inv[c][b];
            }
        }
    }
    double *o = out + q * (int64_t)ND * k;
    if (singular) {
        const double nan = __longlong_as_double(0x7ff8000000000000ll);
        for (int e = 0; e < ND * k; ++e) o[e] = nan;
        if (n_singular) atomicAdd(n_singular, 1ull);
        return;
    }
    for (int j = 0; j < k; ++j) {
        double av[ND], w;
        neighbour(j, av, w);
#pragma unroll
        for (int a = 0; a < ND; ++a) {
            double s = 0.0;
#pragma unroll
            for (int b = 0; b < ND; ++b) s += inv[a][b] * (w * av[b]);
            o[(int64_t)a * k + j] = s;
        }
    }
}

// 1-D KDE: the grid points in ascending order (with their indices), each
// particle adds Kernel(|g - x| / bw) / bw * 4/3 to the points within bw.
__device__ __forceinline__ uint64_t asc_key(double v) {
    const uint64_t b = (uint64_t)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void k_kde_keys(const double *__restrict__ grid, int64_t ng, uint64_t *__restrict__ key,
                           int32_t *__restrict__ idx) {
    const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= ng) return;
    key[g] = asc_key(grid[g]);
    idx[g] = (int32_t)g;
}

__global__ void k_kde_scatter(const double *__restrict__ x, const double *__restrict__ bw, int64_t n,
                              const double *__restrict__ grid, const int32_t *__restrict__ idx, int64_t ng,
                              double *__restrict__ f) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const double d = x[p], b = bw[p];
    // first sorted point >= d - b
    int64_t lo = 0, hi = ng;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (grid[idx[mid]] < d - b)
            lo = mid + 1;
        else
            hi = mid;
    }
    for (int64_t s = lo; s < ng; ++s) {
        const int32_t g = idx[s];
        const double dist = fabs(grid[g] - d);
        if (grid[g] > d + b) break;
        if (dist <= b) atomicAdd(f + g, kernel64(dist / b) / b * 4.0 / 3);
    }
}

}  // namespace mg

using namespace mg;

extern "C" int mg_kernel_weights(const double *ngbdist, const double *h, int64_t nq, int32_t k, double *w,
                                 void *stream_) {
    if (nq < 0 || k < 1 || (nq > 0 && (!ngbdist || !h || !w))) return MG_ERR_ARG;
    if (nq == 0) return MG_OK;
    k_kernel_weights<<<(unsigned)((nq + 127) / 128), 128, 0, as_stream(stream_)>>>(ngbdist, h, nq, k, w);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

template <int DIM, int ORDER>
static void launch_gw(int64_t nq, cudaStream_t st, const double *pos, const int64_t *ngb, int k, const double *h,
                      const int64_t *indices, double box, bool weighted, double *out, unsigned long long *ns) {
    k_gradient_weights<DIM, ORDER><<<(unsigned)((nq + 127) / 128), 128, 0, st>>>(pos, ngb, k, h, indices, nq, box,
                                                                                weighted, out, ns);
}

extern "C" int mg_gradient_weights(const double *pos, int32_t dim, const int64_t *ngb, int32_t k, const double *h,
                                   const int64_t *indices, int64_t nq, double boxsize, int32_t weighted,
                                   int32_t order, double *out, int64_t *n_singular, void *stream_) {
    if (nq < 0 || k < 1 || dim < 1 || dim > 3 || (order != 1 && order != 2)) return MG_ERR_ARG;
    if (nq > 0 && (!pos || !ngb || !h || !indices || !out)) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    if (n_singular) MG_CUDA(cudaMemsetAsync(n_singular, 0, sizeof(int64_t), st));
    if (nq == 0) return MG_OK;
    unsigned long long *ns = reinterpret_cast<unsigned long long *>(n_singular);
    const bool wt = weighted != 0;
    if (order == 1) {
        if (dim == 1) launch_gw<1, 1>(nq, st, pos, ngb, k, h, indices, boxsize, wt, out, ns);
        else if (dim == 2) launch_gw<2, 1>(nq, st, pos, ngb, k, h, indices, boxsize, wt, out, ns);
        else launch_gw<3, 1>(nq, st, pos, ngb, k, h, indices, boxsize, wt, out, ns);
    } else {
        if (dim == 1) launch_gw<1, 2>(nq, st, pos, ngb, k, h, indices, boxsize, wt, out, ns);
        else if (dim == 2) launch_gw<2, 2>(nq, st, pos, ngb, k, h, indices, boxsize, wt, out, ns);
        else launch_gw<3, 2>(nq, st, pos, ngb, k, h, indices, boxsize, wt, out, ns);
    }
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" size_t mg_kde_1d_workspace_bytes(int64_t ng) {
    if (ng < 0) return 0;
    return align_up(sizeof(uint64_t) * (size_t)(ng + 1)) + align_up(sizeof(int32_t) * (size_t)(ng + 1)) +
           radix_sort_workspace_bytes(ng + 1) + 1024;
}

extern "C" int mg_kde_1d(const double *x, const double *bw, int64_t n, const double *grid, int64_t ng, double *f,
                         void *workspace, size_t workspace_bytes, void *stream_) {
    if (n < 0 || ng < 0 || (n > 0 && (!x || !bw)) || (ng > 0 && (!grid || !f))) return MG_ERR_ARG;
    if (ng > 0x7fffffffll) return MG_ERR_UNSUPPORTED;
    if (workspace_bytes < mg_kde_1d_workspace_bytes(ng)) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    if (ng == 0) return MG_OK;
    MG_CUDA(cudaMemsetAsync(f, 0, sizeof(double) * (size_t)ng, st));
    if (n == 0) return MG_OK;
    Carve w(workspace, workspace_bytes);
    uint64_t *key = w.take<uint64_t>((size_t)ng + 1);
    int32_t *idx = w.take<int32_t>((size_t)ng + 1);
    void *sort_ws = w.take<char>(radix_sort_workspace_bytes(ng + 1));
    if (!w.ok()) return MG_ERR_ARG;
    k_kde_keys<<<(unsigned)((ng + 255) / 256), 256, 0, st>>>(grid, ng, key, idx);
    MG_CHECK_LAUNCH();
    int rc = radix_sort_pairs(key, idx, ng, 0, 64, sort_ws, radix_sort_workspace_bytes(ng + 1), st);
    if (rc) return rc;
    k_kde_scatter<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(x, bw, n, grid, idx, ng, f);
    MG_CHECK_LAUNCH();
    return MG_OK;
}
