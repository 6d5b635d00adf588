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
#include "mg_cube.cuh"
#include "mg_scan.cuh"

namespace mg {

constexpr double kKernel3dNorm = 2.546479089470325;  // 8 / pi (kernel3d)
constexpr int kDepWarps = 8;

__device__ __forceinline__ int pmod(int a, int m) { return ((a % m) + m) % m; }

// CubeDiv, cube_div and cube_node (flat node index -> (i, j, l)): mg_cube.cuh

// A particle's node cube: lowest node, counts, offset of the particle from
// the lowest node (node units) and node spacing / h per axis.  The FP64 set-up
// (the reference's divisions and truncations) runs one particle per lane; the
// warp then serves the 32 cubes one after the other, each lane taking its
// cube from the lane that built it.
struct NodeCube {
    int lo[3], cnt[3];
    float u[3], s[3];
};

__device__ __forceinline__ NodeCube shfl_cube(const NodeCube &c, int src) {
    NodeCube r;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        r.lo[d] = __shfl_sync(0xffffffffu, c.lo[d], src);
        r.cnt[d] = __shfl_sync(0xffffffffu, c.cnt[d], src);
        r.u[d] = __shfl_sync(0xffffffffu, c.u[d], src);
        r.s[d] = __shfl_sync(0xffffffffu, c.s[d], src);
    }
    return r;
}

// W(q) with q = |(u - node)| scaled per axis (u: offsets in node units).
__device__ __forceinline__ float cube_w(const float u[3], const float s[3], int i, int j, int l) {
    const float a = (u[0] - (float)i) * s[0], b = (u[1] - (float)j) * s[1], c = (u[2] - (float)l) * s[2];
    return spline_w(sqrtf(fmaf(c, c, fmaf(b, b, a * a))));
}

// GridDensity.  A particle's cube of nodes is usually small (~30 nodes at
// 128^3 over a Plummer sphere) but millions of them share the central nodes,
// so one global atomic per node and particle is contention-bound.  Instead
// each particle's normalisation is found first (warp per particle, no
// atomics), the (8^3-node tile, particle) overlaps are sorted by tile, and one
// CTA per chunk of a tile's overlaps accumulates in shared memory and adds
// each node once.  With a box, a cube that wraps around the grid is deposited
// directly with global atomics (few particles: those within h of the faces).
constexpr int kGdTile = 8;        // nodes per tile side
constexpr int kGdChunk = 4096;    // overlaps per work item
constexpr int kGdWarps = 8;       // warps per work-item CTA
constexpr int kGdOwnNodes = 64;   // cubes up to this many nodes are normalised by their particle's lane

struct GdRange {
    int lo[3], cnt[3];
    float u[3], s;
};

// Node range of particle p (the reference's truncation, clipped without a box).
// The truncations of (x - h) / dx + 1 and (x + h) / dx are decided in FP32
// from the FP32 roundings of x and h (each within ~4e-7 (|x| + h) / dx of
// the FP64 quotients); where either lies within 1e-6 (|x| + h) / dx + 1e-6
// of an integer the FP64 division decides, as in the reference.  FP64
// divisions and conversions run at a small fraction of the FP32 rate on
// this GPU, and this set-up ran twice per particle with ten of them.
__device__ __forceinline__ bool gd_range(const double *__restrict__ pos, const double *__restrict__ h, int64_t p,
                                         const double ctr[3], double size, double dx, double inv_dx, int res,
                                         bool periodic, GdRange &g) {
    const double hs = h[p];
    const float hf = (float)hs, invf = (float)inv_dx;
    bool empty = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double xs = pos[p * 3 + d] - ctr[d] + size / 2 - dx / 2;
        int a, b;
        if (!trunc_pair32((float)xs, hf, invf, a, b)) {
            a = (int)((xs - hs) / dx + 1);
            b = (int)((xs + hs) / dx);
        }
        if (!periodic) {
            a = max(a, 0);
            b = min(b, res - 1);
        }
        g.lo[d] = a;
        g.cnt[d] = b - a + 1;
        empty = empty || g.cnt[d] <= 0;
        g.u[d] = (float)(xs * inv_dx - (double)a);
    }
    g.s = (float)dx / hf;
    return !empty;
}

__device__ __forceinline__ bool gd_inside(const GdRange &g, int res) {
    return g.lo[0] >= 0 && g.lo[1] >= 0 && g.lo[2] >= 0 && g.lo[0] + g.cnt[0] <= res && g.lo[1] + g.cnt[1] <= res &&
           g.lo[2] + g.cnt[2] <= res;
}

__device__ __forceinline__ uint32_t gd_tiles(const GdRange &g) {
    uint32_t t = 1;
#pragma unroll
    for (int d = 0; d < 3; ++d) t *= (uint32_t)((g.lo[d] + g.cnt[d] - 1) / kGdTile - g.lo[d] / kGdTile + 1);
    return t;
}

// count != 0: only the number of tile overlaps (an upper bound of the pairs),
// summed into *npairs.  Otherwise: normalisation, direct deposit of wrapping
// cubes, per-particle data of the rest and their overlap counts.
__global__ __launch_bounds__(kDepWarps * 32) void k_gd_prep(const double *__restrict__ pos,
                                                           const double *__restrict__ h,
                                                           const double *__restrict__ f, int64_t n, double cx,
                                                           double cy, double cz, double size, int res, bool periodic,
                                                           bool count, unsigned long long *__restrict__ npairs,
                                                           uint32_t *__restrict__ tcount, float4 *__restrict__ pu,
                                                           int4 *__restrict__ plo, int4 *__restrict__ pcnt,
                                                           double *__restrict__ pfac, double *__restrict__ grid,
                                                           int64_t *__restrict__ n_skipped) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * kDepWarps;
    const double dx = size / (double)(res - 1), inv_dx = 1.0 / dx;
    const double inv_vol = 1.0 / (dx * dx * dx);
    const double ctr[3] = {cx, cy, cz};
    unsigned long long counted = 0;
    for (int64_t p0 = ((int64_t)blockIdx.x * kDepWarps + (threadIdx.x >> 5)) * 32; p0 < n; p0 += nwarps * 32) {
        // lane: FP64 set-up of particle p0 + lane
        const int64_t pl = p0 + lane;
        GdRange gr;
        const bool anyl = pl < n && gd_range(pos, h, pl, ctr, size, dx, inv_dx, res, periodic, gr);
        const bool insidel = anyl && gd_inside(gr, res);
        if (count) {
            if (insidel) counted += gd_tiles(gr);
            continue;
        }
        NodeCube gl;
        if (anyl) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                gl.lo[d] = gr.lo[d];
                gl.cnt[d] = gr.cnt[d];
                gl.u[d] = gr.u[d];
                gl.s[d] = gr.s;
            }
        }
        const unsigned anym = __ballot_sync(0xffffffffu, anyl), insm = __ballot_sync(0xffffffffu, insidel);
        uint32_t my_tiles = 0;
        // A lane normalises its own particle when the cube is small (the
        // usual case: ~30 nodes at 128^3 over a Plummer sphere); the warp
        // takes the large cubes and those that wrap around the box one
        // particle after another (a chain of shuffles, loop and reduction
        // per particle, too serial for the small ones).
        bool own = false;
        if (insidel && (int64_t)gr.cnt[0] * gr.cnt[1] * gr.cnt[2] <= kGdOwnNodes) {
            own = true;
            const float s3[3] = {gr.s, gr.s, gr.s};
            float ws = 0.0f;
            for (int i = 0; i < gr.cnt[0]; ++i)
                for (int jj = 0; jj < gr.cnt[1]; ++jj)
                    for (int l = 0; l < gr.cnt[2]; ++l) ws += cube_w(gr.u, s3, i, jj, l);
            if (ws > 0.0f) {
                my_tiles = gd_tiles(gr);
                pu[pl] = make_float4(gr.u[0], gr.u[1], gr.u[2], gr.s);
                plo[pl] = make_int4(gr.lo[0], gr.lo[1], gr.lo[2], 0);
                pcnt[pl] = make_int4(gr.cnt[0], gr.cnt[1], gr.cnt[2], 0);
                pfac[pl] = f[pl] / (double)ws * inv_vol;
            }
        }
        const unsigned ownm = __ballot_sync(0xffffffffu, own);
        for (int k = 0; k < 32; ++k) {
            if (!(anym >> k & 1u) || (ownm >> k & 1u)) continue;
            const int64_t p = p0 + k;
            const NodeCube g = shfl_cube(gl, k);
            const bool inside = insm >> k & 1u;
            if (!inside && (g.cnt[0] > 4 * res + 8 || g.cnt[1] > 4 * res + 8 || g.cnt[2] > 4 * res + 8)) {
                // with a box the range is not clipped: a cube spanning the grid
                // many times over (h far beyond the box) is refused
                if (lane == 0 && n_skipped) atomicAdd((unsigned long long *)n_skipped, 1ull);
                continue;
            }
            const int64_t total = (int64_t)g.cnt[0] * g.cnt[1] * g.cnt[2];
            const CubeDiv cd = cube_div(g.cnt[1], g.cnt[2], total);
            float wsum = 0.0f;
            for (int64_t c = lane; c < total; c += 32) {
                int i, j, l;
                cube_node(c, cd, i, j, l);
                wsum += cube_w(g.u, g.s, i, j, l);
            }
            wsum = warp_sum(wsum);
            if (!(wsum > 0.0f)) continue;
            // one lane divides (a warp-wide FP64 division is 32 of them, and
            // FP64 runs at a small fraction of the FP32 rate on this GPU)
            double fac = 0.0;
            if (lane == 0) fac = f[p] / (double)wsum * inv_vol;
            fac = __shfl_sync(0xffffffffu, fac, 0);
            if (inside) {
                if (lane == k) {
                    my_tiles = gd_tiles(gr);
                    pu[p] = make_float4(gr.u[0], gr.u[1], gr.u[2], gr.s);
                    plo[p] = make_int4(gr.lo[0], gr.lo[1], gr.lo[2], 0);
                    pcnt[p] = make_int4(gr.cnt[0], gr.cnt[1], gr.cnt[2], 0);
                    pfac[p] = fac;
                }
            } else {
                for (int64_t c = lane; c < total; c += 32) {
                    int i, j, l;
                    cube_node(c, cd, i, j, l);
                    const float w = cube_w(g.u, g.s, i, j, l);
                    if (w == 0.0f) continue;
                    const int gx = pmod(g.lo[0] + i, res), gy = pmod(g.lo[1] + j, res), gz = pmod(g.lo[2] + l, res);
                    atomicAdd(grid + ((int64_t)gx * res + gy) * res + gz, fac * (double)w);
                }
            }
        }
        if (pl < n) tcount[pl] = my_tiles;
    }
    counted = warp_sum(counted);
    if (count && lane == 0 && counted) atomicAdd(npairs, counted);
}

// overlaps of particle p at [toff[p], toff[p + 1]) (none: deposited directly or nothing)
__global__ void k_gd_pairs(const int4 *__restrict__ plo, const int4 *__restrict__ pcnt,
                           const uint32_t *__restrict__ toff, int64_t n, int ntx, uint64_t *__restrict__ key,
                           int32_t *__restrict__ val) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n || toff[p + 1] == toff[p]) return;
    const int4 lo = plo[p], cn = pcnt[p];
    int64_t e = toff[p];
    for (int tx = lo.x / kGdTile; tx <= (lo.x + cn.x - 1) / kGdTile; ++tx)
        for (int ty = lo.y / kGdTile; ty <= (lo.y + cn.y - 1) / kGdTile; ++ty)
            for (int tz = lo.z / kGdTile; tz <= (lo.z + cn.z - 1) / kGdTile; ++tz, ++e) {
                key[e] = ((uint64_t)((tx * ntx + ty) * ntx + tz) << 32) | (uint64_t)p;
                val[e] = (int32_t)p;
            }
}

// tile t's overlaps are [tbeg[t], tbeg[t + 1]) of the sorted pairs; items of
// at most kGdChunk overlaps
__global__ void k_gd_tile_starts(const uint64_t *__restrict__ key, int64_t npairs, int ntiles,
                                 uint32_t *__restrict__ tbeg) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e > npairs) return;
    // unused tail entries carry all-ones keys: beyond the last tile
    const int t = e < npairs ? (int)min(key[e] >> 32, (uint64_t)ntiles) : ntiles;
    const int tp = e > 0 ? (int)min(key[e - 1] >> 32, (uint64_t)ntiles) : -1;
    for (int u = tp + 1; u <= t; ++u) tbeg[u] = (uint32_t)e;
}

__global__ void k_gd_item_count(const uint32_t *__restrict__ tbeg, int ntiles, uint32_t *__restrict__ icount) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < ntiles) icount[t] = (tbeg[t + 1] - tbeg[t] + kGdChunk - 1) / kGdChunk;
    if (t == ntiles) icount[t] = 0;
}

__global__ void k_gd_items(const uint32_t *__restrict__ tbeg, const uint32_t *__restrict__ ioff, int ntiles,
                           int4 *__restrict__ items) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntiles) return;
    const uint32_t b = tbeg[t], e = tbeg[t + 1];
    uint32_t it = ioff[t];
    for (uint32_t s = b; s < e; s += kGdChunk, ++it) items[it] = make_int4(t, (int)s, (int)min(e, s + kGdChunk), 0);
}

__global__ __launch_bounds__(kGdWarps * 32) void k_gd_tile(const int4 *__restrict__ items,
                                                          const uint32_t *__restrict__ nitems,
                                                          const int32_t *__restrict__ val,
                                                          const float4 *__restrict__ pu, const int4 *__restrict__ plo,
                                                          const int4 *__restrict__ pcnt,
                                                          const double *__restrict__ pfac, int res,
                                                          double *__restrict__ grid) {
    __shared__ float acc[kGdTile * kGdTile * kGdTile];
    const int item = blockIdx.x;
    if (item >= (int)*nitems) return;
    const int4 it = items[item];
    const int ntx = (res + kGdTile - 1) / kGdTile;
    const int t0 = it.x / (ntx * ntx), t1 = (it.x / ntx) % ntx, t2 = it.x % ntx;
    const int base[3] = {t0 * kGdTile, t1 * kGdTile, t2 * kGdTile};
    for (int c = threadIdx.x; c < kGdTile * kGdTile * kGdTile; c += blockDim.x) acc[c] = 0.0f;
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    for (int e = it.y + wib; e < it.z; e += kGdWarps) {
        const int p = val[e];
        const float4 u4 = pu[p];
        const int4 lo = plo[p], cn = pcnt[p];
        const float u[3] = {u4.x, u4.y, u4.z}, s3[3] = {u4.w, u4.w, u4.w};
        const float fac = (float)pfac[p];
        // the cube's nodes inside this tile
        const int a0 = max(lo.x, base[0]), b0 = min(lo.x + cn.x, base[0] + kGdTile);
        const int a1 = max(lo.y, base[1]), b1 = min(lo.y + cn.y, base[1] + kGdTile);
        const int a2 = max(lo.z, base[2]), b2 = min(lo.z + cn.z, base[2] + kGdTile);
        const int n1 = b1 - a1, n2 = b2 - a2, nn = (b0 - a0) * n1 * n2;
        const CubeDiv cd = cube_div(n1, n2, nn);
        for (int c = lane; c < nn; c += 32) {
            int i, j, l;
            cube_node(c, cd, i, j, l);
            const int gx = a0 + i, gy = a1 + j, gz = a2 + l;
            const float w = cube_w(u, s3, gx - lo.x, gy - lo.y, gz - lo.z);
            if (w != 0.0f)
                atomicAdd(&acc[((gx - base[0]) * kGdTile + (gy - base[1])) * kGdTile + (gz - base[2])], fac * w);
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < kGdTile * kGdTile * kGdTile; c += blockDim.x) {
        const float v = acc[c];
        if (v == 0.0f) continue;
        const int gx = base[0] + c / (kGdTile * kGdTile), gy = base[1] + (c / kGdTile) % kGdTile,
                  gz = base[2] + c % kGdTile;
        if (gx < res && gy < res && gz < res) atomicAdd(grid + ((int64_t)gx * res + gy) * res + gz, (double)v);
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
    for (int64_t p0 = ((int64_t)blockIdx.x * kDepWarps + (threadIdx.x >> 5)) * 32; p0 < n; p0 += nwarps * 32) {
        // lane: set-up of particle p0 + lane
        const int64_t pl = p0 + lane;
        NodeCube gl;
        bool ok = false;
        double facl = 0.0;
        if (pl < n) {
            const double hs = h[pl], hzs = hz[pl];
            const double xs[3] = {pos[pl * 3 + 0] - cx + size_xy / 2, pos[pl * 3 + 1] - cy + size_xy / 2,
                                  z[pl] - cz + size_z / 2};
            const double sp[3] = {dx, dx, dz}, hh[3] = {hs, hs, hzs};
            const int rr[3] = {res_xy, res_xy, res_z};
            ok = true;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const int a = max((int)((xs[d] - hh[d]) / sp[d] + 1), 0),
                          b = min((int)((xs[d] + hh[d]) / sp[d]), rr[d] - 1);
                gl.lo[d] = a;
                gl.cnt[d] = b - a + 1;
                ok = ok && gl.cnt[d] > 0;
                gl.u[d] = (float)(xs[d] / sp[d] - (double)a);
                gl.s[d] = (float)(sp[d] / hh[d]);
            }
            facl = kKernel3dNorm * f[pl] / (hs * hs * hzs);
        }
        const unsigned okm = __ballot_sync(0xffffffffu, ok);
        for (int k = 0; k < 32; ++k) {
            if (!(okm >> k & 1u)) continue;
            const NodeCube g = shfl_cube(gl, k);
            const double fac = __shfl_sync(0xffffffffu, facl, k);
            const int64_t total = (int64_t)g.cnt[0] * g.cnt[1] * g.cnt[2];
            const CubeDiv cd = cube_div(g.cnt[1], g.cnt[2], total);
            for (int64_t c = lane; c < total; c += 32) {
                int i, j, l;
                cube_node(c, cd, i, j, l);
                const float w = cube_w(g.u, g.s, i, j, l);
                if (w == 0.0f) continue;
                atomicAdd(grid + ((int64_t)(g.lo[0] + i) * res_xy + (g.lo[1] + j)) * res_z + (g.lo[2] + l),
                          fac * (double)w);
            }
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
    for (int64_t p0 = ((int64_t)blockIdx.x * kDepWarps + (threadIdx.x >> 5)) * 32; p0 < n; p0 += nwarps * 32) {
        const int64_t pl = p0 + lane;
        NodeCube gl;
        bool ok = false;
        if (pl < n) {
            const double hs = h[pl], hs_dx = hs / dx;
            ok = true;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const double xs = pos[pl * 3 + d] - ctr[d];
                const double gi = (xs + size / 2) / dx - 0.5;
                const int a = max((int)(gi - hs_dx + 1), 0), b = min((int)(gi + hs_dx), res - 1);
                gl.lo[d] = a;
                gl.cnt[d] = b - a + 1;
                ok = ok && gl.cnt[d] > 0;
                gl.u[d] = (float)((xs - start) / step - (double)a);
                gl.s[d] = (float)(step / hs);
            }
        }
        const unsigned okm = __ballot_sync(0xffffffffu, ok);
        for (int k = 0; k < 32; ++k) {
            if (!(okm >> k & 1u)) continue;
            const int64_t p = p0 + k;
            const NodeCube g = shfl_cube(gl, k);
            const int64_t total = (int64_t)g.cnt[0] * g.cnt[1] * g.cnt[2];
            const CubeDiv cd = cube_div(g.cnt[1], g.cnt[2], total);
            float wsum = 0.0f;
            for (int64_t c = lane; c < total; c += 32) {
                int i, j, l;
                cube_node(c, cd, i, j, l);
                wsum += cube_w(g.u, g.s, i, j, l);
            }
            wsum = warp_sum(wsum);
            if (!(wsum > 0.0f)) continue;
            double wfac = 0.0;  // one lane divides (see k_gd_prep)
            if (lane == 0) wfac = wt[p] / (double)wsum;
            wfac = __shfl_sync(0xffffffffu, wfac, 0);
            const double ffac = f[p] * wfac;
            for (int64_t c = lane; c < total; c += 32) {
                int i, j, l;
                cube_node(c, cd, i, j, l);
                const float w = cube_w(g.u, g.s, i, j, l);
                if (w == 0.0f) continue;
                const int64_t cell = ((int64_t)(g.lo[0] + i) * res + (g.lo[1] + j)) * res + (g.lo[2] + l);
                atomicAdd(num + cell, ffac * (double)w);
                atomicAdd(den + cell, wfac * (double)w);
            }
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

extern "C" int mg_grid_density_count(const double *pos, const double *h, int64_t n, double cx, double cy,
                                     double cz, double size, int32_t res, int32_t periodic, int64_t *npairs,
                                     void *stream_) {
    if (!npairs || n < 0 || res < 2 || !(size > 0.0) || (n > 0 && (!pos || !h))) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    MG_CUDA(cudaMemsetAsync(npairs, 0, sizeof(int64_t), st));
    if (n == 0) return MG_OK;
    k_gd_prep<<<dep_blocks(n), kDepWarps * 32, 0, st>>>(pos, h, nullptr, n, cx, cy, cz, size, res, periodic != 0, true,
                                                       reinterpret_cast<unsigned long long *>(npairs), nullptr, nullptr,
                                                       nullptr, nullptr, nullptr, nullptr, nullptr);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

static int gd_ntiles(int res) {
    const int ntx = (res + kGdTile - 1) / kGdTile;
    return ntx * ntx * ntx;
}

extern "C" size_t mg_grid_density_workspace_bytes(int64_t n, int64_t npairs, int32_t res) {
    if (n < 0 || npairs < 0 || res < 2) return 0;
    const int nt = gd_ntiles(res);
    const int64_t maxit = (int64_t)nt + npairs / kGdChunk + 1;
    return align_up(sizeof(uint32_t) * (size_t)(n + 1)) + align_up(scan_workspace_bytes(n + 1)) +
           align_up(sizeof(float4) * (size_t)(n + 1)) + 2 * align_up(sizeof(int4) * (size_t)(n + 1)) +
           align_up(sizeof(double) * (size_t)(n + 1)) + align_up(sizeof(uint64_t) * (size_t)(npairs + 1)) +
           align_up(sizeof(int32_t) * (size_t)(npairs + 1)) + radix_sort_workspace_bytes(npairs + 1) +
           3 * align_up(sizeof(uint32_t) * (size_t)(nt + 2)) + align_up(scan_workspace_bytes(nt + 1)) +
           align_up(sizeof(int4) * (size_t)maxit) + 4096;
}

extern "C" int mg_grid_density(const double *pos, const double *h, const double *f, int64_t n, double cx, double cy,
                               double cz, double size, int32_t res, int32_t periodic, double *grid,
                               int64_t *n_skipped, int64_t npairs, void *workspace, size_t workspace_bytes,
                               void *stream_) {
    if (!grid || n < 0 || res < 2 || !(size > 0.0) || npairs < 0 || (n > 0 && (!pos || !h || !f))) return MG_ERR_ARG;
    if (n > 0x7fffffffll || npairs > 0x7fffffffll) return MG_ERR_UNSUPPORTED;
    if (workspace_bytes < mg_grid_density_workspace_bytes(n, npairs, res)) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    const int64_t cells = (int64_t)res * res * res;
    MG_CUDA(cudaMemsetAsync(grid, 0, sizeof(double) * (size_t)cells, st));
    if (n_skipped) MG_CUDA(cudaMemsetAsync(n_skipped, 0, sizeof(int64_t), st));
    if (n == 0) return MG_OK;
    const int nt = gd_ntiles(res), ntx = (res + kGdTile - 1) / kGdTile;
    const int64_t maxit = (int64_t)nt + npairs / kGdChunk + 1;
    Carve w(workspace, workspace_bytes);
    uint32_t *tcount = w.take<uint32_t>((size_t)n + 1);
    void *scan_ws = w.take<char>(scan_workspace_bytes(n + 1));
    float4 *pu = w.take<float4>((size_t)n + 1);
    int4 *plo = w.take<int4>((size_t)n + 1);
    int4 *pcnt = w.take<int4>((size_t)n + 1);
    double *pfac = w.take<double>((size_t)n + 1);
    uint64_t *key = w.take<uint64_t>((size_t)npairs + 1);
    int32_t *val = w.take<int32_t>((size_t)npairs + 1);
    void *sort_ws = w.take<char>(radix_sort_workspace_bytes(npairs + 1));
    uint32_t *tbeg = w.take<uint32_t>((size_t)nt + 2);
    uint32_t *ioff = w.take<uint32_t>((size_t)nt + 2);
    uint32_t *nitems = w.take<uint32_t>((size_t)nt + 2);
    void *scan_ws2 = w.take<char>(scan_workspace_bytes(nt + 1));
    int4 *items = w.take<int4>((size_t)maxit);
    if (!w.ok()) return MG_ERR_ARG;
    // 1. normalisation, direct deposits of wrapping cubes, overlap counts
    k_gd_prep<<<dep_blocks(n), kDepWarps * 32, 0, st>>>(pos, h, f, n, cx, cy, cz, size, res, periodic != 0, false,
                                                       nullptr, tcount, pu, plo, pcnt, pfac, grid, n_skipped);
    MG_CHECK_LAUNCH();
    MG_CUDA(cudaMemsetAsync(tcount + n, 0, sizeof(uint32_t), st));
    int rc = exclusive_scan_u32(tcount, tcount, n + 1, scan_ws, st);  // -> offsets
    if (rc) return rc;
    // 2. (tile, particle) overlaps sorted by tile; the counted bound may exceed
    //    the overlaps made, and the rest of the buffer sorts last
    if (npairs == 0) return MG_OK;
    MG_CUDA(cudaMemsetAsync(key, 0xff, sizeof(uint64_t) * (size_t)npairs, st));
    k_gd_pairs<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(plo, pcnt, tcount, n, ntx, key, val);
    MG_CHECK_LAUNCH();
    int tile_bits = 1;
    while ((1 << tile_bits) < nt + 1) ++tile_bits;
    rc = radix_sort_pairs(key, val, npairs, 32, tile_bits + 1, sort_ws, radix_sort_workspace_bytes(npairs + 1), st);
    if (rc) return rc;
    // 3. work items of at most kGdChunk overlaps of one tile
    MG_CUDA(cudaMemsetAsync(tbeg, 0, sizeof(uint32_t) * ((size_t)nt + 1), st));
    k_gd_tile_starts<<<(unsigned)((npairs + 1 + 255) / 256), 256, 0, st>>>(key, npairs, nt, tbeg);
    MG_CHECK_LAUNCH();
    k_gd_item_count<<<(unsigned)((nt + 1 + 255) / 256), 256, 0, st>>>(tbeg, nt, ioff);
    MG_CHECK_LAUNCH();
    rc = exclusive_scan_u32(ioff, ioff, nt + 1, scan_ws2, st);
    if (rc) return rc;
    MG_CUDA(cudaMemcpyAsync(nitems, ioff + nt, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    k_gd_items<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(tbeg, ioff, nt, items);
    MG_CHECK_LAUNCH();
    // 4. shared-memory accumulation per item, one global add per node
    k_gd_tile<<<(unsigned)maxit, kGdWarps * 32, 0, st>>>(items, nitems, val, pu, plo, pcnt, pfac, res, grid);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" int mg_ppz_cube(const double *pos, const double *h, const double *f, const double *z, const double *hz,
                           int64_t n, double cx, double cy, double cz, double size_xy, double size_z, int32_t res_xy,
                           int32_t res_z, double *grid, void *stream_) {
    if (!grid || n < 0 || res_xy < 2 || res_z < 2 || !(size_xy > 0.0) || !(size_z > 0.0) ||
        (n > 0 && (!pos || !h || !f || !z || !hz)))
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
    if (!result || !weight || n < 0 || res < 2 || !(size > 0.0) || (n > 0 && (!pos || !h || !f || !wt)))
        return MG_ERR_ARG;
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
