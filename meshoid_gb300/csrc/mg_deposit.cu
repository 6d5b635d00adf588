// 3-D deposition onto Cartesian grids:
//   mg_grid_density       GridDensity            src/meshoid/grid_deposition.py:534-600
//                         (Meshoid.DepositToGrid src/meshoid/Meshoid.py:557-593)
//   mg_ppz_cube           Grid_PPZ_DataCube      src/meshoid/grid_deposition.py:339-392
//   mg_weighted_interp3d  WeightedGridInterp3D   src/meshoid/grid_deposition.py:439-531
//
// One warp per particle (grid-stride over particles).  The node range of a
// particle is computed from its FP64 position with the reference's own
// expressions (C truncation, the same clipping or periodic wrap), so every
// particle touches exactly the reference's nodes.  Kernel weights are FP32:
// the particle's offset from its lowest node is taken in FP64 in node units
// and rounded once, so q carries ~1e-7 relative error.  The normalising sums
// (GridDensity, WeightedGridInterp3D) are warp reductions; the deposits are
// FP64 atomics into the caller's grid (summation order, hence the last bits,
// varies between runs).
#include "mg_common.cuh"

namespace mg {

constexpr double kKernel3dNorm = 2.546479089470325;  // 8 / pi (kernel3d)
constexpr int kDepWarps = 8;

__device__ __forceinline__ int pmod(int a, int m) { return ((a % m) + m) % m; }

// Node (i, j, l) of a cube of ny * nz columns from a flat index.
__device__ __forceinline__ void cube_node(int64_t c, int ny, int nz, int &i, int &j, int &l) {
    const int64_t col = c / nz;
    l = (int)(c - col * nz);
    i = (int)(col / ny);
    j = (int)(col - (int64_t)i * ny);
}

// W(q) with q = |(u - node)| scaled per axis (u: offsets in node units).
__device__ __forceinline__ float cube_w(const float u[3], const float s[3], int i, int j, int l) {
    const float a = (u[0] - (float)i) * s[0], b = (u[1] - (float)j) * s[1], c = (u[2] - (float)l) * s[2];
    return spline_w(sqrtf(fmaf(c, c, fmaf(b, b, a * a))));
}

__global__ __launch_bounds__(kDepWarps * 32) void k_grid_density(const double *__restrict__ pos,
                                                                const double *__restrict__ h,
                                                                const double *__restrict__ f, int64_t n, double cx,
                                                                double cy, double cz, double size, int res,
                                                                bool periodic, double *__restrict__ grid,
                                                                int64_t *__restrict__ n_skipped) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * kDepWarps;
    const double dx = size / (double)(res - 1);
    const double inv_vol = 1.0 / (dx * dx * dx);
    const double ctr[3] = {cx, cy, cz};
    for (int64_t p = (int64_t)blockIdx.x * kDepWarps + (threadIdx.x >> 5); p < n; p += nwarps) {
        const double hs = h[p];
        int lo[3], cnt[3];
        float u[3], s[3];
        bool empty = false;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double xs = pos[p * 3 + d] - ctr[d] + size / 2 - dx / 2;
            int a = (int)((xs - hs) / dx + 1), b = (int)((xs + hs) / dx);
            if (!periodic) {
                a = max(a, 0);
                b = min(b, res - 1);
            }
            lo[d] = a;
            cnt[d] = b - a + 1;
            empty = empty || cnt[d] <= 0;
            u[d] = (float)(xs / dx - (double)a);
            s[d] = (float)(dx / hs);
        }
        if (empty) continue;
        // with a box the range is not clipped: a cube spanning the grid many
        // times over (h far beyond the box) is refused rather than looped over
        if (cnt[0] > 4 * res + 8 || cnt[1] > 4 * res + 8 || cnt[2] > 4 * res + 8) {
            if (lane == 0 && n_skipped) atomicAdd((unsigned long long *)n_skipped, 1ull);
            continue;
        }
        const int64_t total = (int64_t)cnt[0] * cnt[1] * cnt[2];
        float wsum = 0.0f;
        for (int64_t c = lane; c < total; c += 32) {
            int i, j, l;
            cube_node(c, cnt[1], cnt[2], i, j, l);
            wsum += cube_w(u, s, i, j, l);
        }
        wsum = warp_sum(wsum);
        if (!(wsum > 0.0f)) continue;
        const double fac = f[p] / (double)wsum * inv_vol;
        for (int64_t c = lane; c < total; c += 32) {
            int i, j, l;
            cube_node(c, cnt[1], cnt[2], i, j, l);
            const float w = cube_w(u, s, i, j, l);
            if (w == 0.0f) continue;
            const int gx = pmod(lo[0] + i, res), gy = pmod(lo[1] + j, res), gz = pmod(lo[2] + l, res);
            atomicAdd(grid + ((int64_t)gx * res + gy) * res + gz, fac * (double)w);
        }
    }
}

__global__ __launch_bounds__(kDepWarps * 32) void k_ppz_cube(const double *__restrict__ pos,
                                                            const double *__restrict__ h,
                                                            const double *__restrict__ f,
                                                            const double *__restrict__ z,
                                                            const double *__restrict__ hz, int64_t n, double cx,
                                                            double cy, double cz, double size_xy, double size_z,
                                                            int res_xy, int res_z, double *__restrict__ grid) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * kDepWarps;
    const double dx = size_xy / (double)(res_xy - 1), dz = size_z / (double)(res_z - 1);
    for (int64_t p = (int64_t)blockIdx.x * kDepWarps + (threadIdx.x >> 5); p < n; p += nwarps) {
        const double hs = h[p], hzs = hz[p];
        const double xs[3] = {pos[p * 3 + 0] - cx + size_xy / 2, pos[p * 3 + 1] - cy + size_xy / 2,
                              z[p] - cz + size_z / 2};
        const double sp[3] = {dx, dx, dz}, hh[3] = {hs, hs, hzs};
        const int rr[3] = {res_xy, res_xy, res_z};
        int lo[3], cnt[3];
        float u[3], s[3];
        bool empty = false;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int a = max((int)((xs[d] - hh[d]) / sp[d] + 1), 0), b = min((int)((xs[d] + hh[d]) / sp[d]), rr[d] - 1);
            lo[d] = a;
            cnt[d] = b - a + 1;
            empty = empty || cnt[d] <= 0;
            u[d] = (float)(xs[d] / sp[d] - (double)a);
            s[d] = (float)(sp[d] / hh[d]);
        }
        if (empty) continue;
        const double fac = kKernel3dNorm * f[p] / (hs * hs * hzs);
        const int64_t total = (int64_t)cnt[0] * cnt[1] * cnt[2];
        for (int64_t c = lane; c < total; c += 32) {
            int i, j, l;
            cube_node(c, cnt[1], cnt[2], i, j, l);
            const float w = cube_w(u, s, i, j, l);
            if (w == 0.0f) continue;
            atomicAdd(grid + ((int64_t)(lo[0] + i) * res_xy + (lo[1] + j)) * res_z + (lo[2] + l), fac * (double)w);
        }
    }
}

__global__ __launch_bounds__(kDepWarps * 32) void k_weighted_interp3d(const double *__restrict__ pos,
                                                                     const double *__restrict__ h,
                                                                     const double *__restrict__ f,
                                                                     const double *__restrict__ wt, int64_t n,
                                                                     double cx, double cy, double cz, double size,
                                                                     int res, double *__restrict__ num,
                                                                     double *__restrict__ den) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * kDepWarps;
    const double dx = size / (double)(res - 1);
    // cell-centre nodes: linspace(dx/2 - size/2, size/2 - dx/2, res)
    const double start = dx / 2 - size / 2, stop = size / 2 - dx / 2;
    const double step = (stop - start) / (double)(res - 1);
    const double ctr[3] = {cx, cy, cz};
    for (int64_t p = (int64_t)blockIdx.x * kDepWarps + (threadIdx.x >> 5); p < n; p += nwarps) {
        const double hs = h[p], hs_dx = hs / dx;
        int lo[3], cnt[3];
        float u[3], s[3];
        bool empty = false;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double xs = pos[p * 3 + d] - ctr[d];
            const double gi = (xs + size / 2) / dx - 0.5;
            const int a = max((int)(gi - hs_dx + 1), 0), b = min((int)(gi + hs_dx), res - 1);
            lo[d] = a;
            cnt[d] = b - a + 1;
            empty = empty || cnt[d] <= 0;
            u[d] = (float)((xs - start) / step - (double)a);
            s[d] = (float)(step / hs);
        }
        if (empty) continue;
        const int64_t total = (int64_t)cnt[0] * cnt[1] * cnt[2];
        float wsum = 0.0f;
        for (int64_t c = lane; c < total; c += 32) {
            int i, j, l;
            cube_node(c, cnt[1], cnt[2], i, j, l);
            wsum += cube_w(u, s, i, j, l);
        }
        wsum = warp_sum(wsum);
        if (!(wsum > 0.0f)) continue;
        const double wfac = wt[p] / (double)wsum, ffac = f[p] * wfac;
        for (int64_t c = lane; c < total; c += 32) {
            int i, j, l;
            cube_node(c, cnt[1], cnt[2], i, j, l);
            const float w = cube_w(u, s, i, j, l);
            if (w == 0.0f) continue;
            const int64_t cell = ((int64_t)(lo[0] + i) * res + (lo[1] + j)) * res + (lo[2] + l);
            atomicAdd(num + cell, ffac * (double)w);
            atomicAdd(den + cell, wfac * (double)w);
        }
    }
}

// result = num / den; NaN where no weight arrived (the caller fills those
// cells with the nearest particle's value); counts them.
__global__ void k_interp_finish(const double *__restrict__ den, double *__restrict__ res_grid, int64_t cells,
                                int64_t *__restrict__ n_empty) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    bool e = false;
    if (c < cells) {
        const double d = den[c];
        e = d == 0.0;
        res_grid[c] = e ? __longlong_as_double(0x7ff8000000000000ll) : res_grid[c] / d;
    }
    const unsigned m = __ballot_sync(0xffffffffu, e);
    if ((threadIdx.x & 31) == 0 && m && n_empty) atomicAdd((unsigned long long *)n_empty, (unsigned long long)__popc(m));
}

static unsigned dep_blocks(int64_t n) {
    int dev = 0, nsm = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t need = (n + kDepWarps - 1) / kDepWarps;
    const int64_t cap = (int64_t)nsm * 16;
    return (unsigned)(need < cap ? need : cap);
}

}  // namespace mg

using namespace mg;

extern "C" int mg_grid_density(const double *pos, const double *h, const double *f, int64_t n, double cx, double cy,
                               double cz, double size, int32_t res, int32_t periodic, double *grid,
                               int64_t *n_skipped, void *stream_) {
    if (!pos || !h || !f || !grid || n < 0 || res < 2 || !(size > 0.0)) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    const int64_t cells = (int64_t)res * res * res;
    MG_CUDA(cudaMemsetAsync(grid, 0, sizeof(double) * (size_t)cells, st));
    if (n_skipped) MG_CUDA(cudaMemsetAsync(n_skipped, 0, sizeof(int64_t), st));
    if (n == 0) return MG_OK;
    k_grid_density<<<dep_blocks(n), kDepWarps * 32, 0, st>>>(pos, h, f, n, cx, cy, cz, size, res, periodic != 0,
                                                            grid, n_skipped);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" int mg_ppz_cube(const double *pos, const double *h, const double *f, const double *z, const double *hz,
                           int64_t n, double cx, double cy, double cz, double size_xy, double size_z, int32_t res_xy,
                           int32_t res_z, double *grid, void *stream_) {
    if (!pos || !h || !f || !z || !hz || !grid || n < 0 || res_xy < 2 || res_z < 2 || !(size_xy > 0.0) ||
        !(size_z > 0.0))
        return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    const int64_t cells = (int64_t)res_xy * res_xy * res_z;
    MG_CUDA(cudaMemsetAsync(grid, 0, sizeof(double) * (size_t)cells, st));
    if (n == 0) return MG_OK;
    k_ppz_cube<<<dep_blocks(n), kDepWarps * 32, 0, st>>>(pos, h, f, z, hz, n, cx, cy, cz, size_xy, size_z, res_xy,
                                                        res_z, grid);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" int mg_weighted_interp3d(const double *pos, const double *h, const double *f, const double *wt,
                                    int64_t n, double cx, double cy, double cz, double size, int32_t res,
                                    double *result, double *weight, int64_t *n_empty, void *stream_) {
    if (!pos || !h || !f || !wt || !result || !weight || n < 0 || res < 2 || !(size > 0.0)) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    const int64_t cells = (int64_t)res * res * res;
    MG_CUDA(cudaMemsetAsync(result, 0, sizeof(double) * (size_t)cells, st));
    MG_CUDA(cudaMemsetAsync(weight, 0, sizeof(double) * (size_t)cells, st));
    if (n_empty) MG_CUDA(cudaMemsetAsync(n_empty, 0, sizeof(int64_t), st));
    if (n > 0) {
        k_weighted_interp3d<<<dep_blocks(n), kDepWarps * 32, 0, st>>>(pos, h, f, wt, n, cx, cy, cz, size, res,
                                                                     result, weight);
        MG_CHECK_LAUNCH();
    }
    k_interp_finish<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(weight, result, cells, n_empty);
    MG_CHECK_LAUNCH();
    return MG_OK;
}
