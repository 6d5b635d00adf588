// Emission/absorption ray tracing along the z sightlines of a pixel grid:
// radtransfer_singlethread (src/meshoid/radiation/radtransfer.py:87-200).
//
// Per pixel the reference walks the particles from the largest z to the
// smallest (relative to the centre) and applies, for every particle whose
// footprint holds the pixel, I <- exp(-tau) I - expm1(-tau) S with tau =
// kappa kernel2d(r/h) m/h^2 and S = j / (4 pi kappa + 1e-100).  The walk is
// ordered, so here:
//   1. particles are sorted by z, descending (stable radix sort of the FP64
//      bits: ties by index);
//   2. every (32 x 32-pixel tile, particle) overlap becomes a pair, generated
//      in z order and stably sorted by tile, so each tile's list is in z order;
//   3. a tile's list is cut into chunks of kRtChunk; one CTA per chunk walks it
//      from I = 0, tau = 0 for the tile's 1024 pixels (4 per thread, FP32);
//   4. the chunks of a tile are composed front to back: I = sum_c I_c
//      exp(-sum of tau in front of c) + i0 exp(-tau_total) — exact, since the
//      attenuation of a chunk is the product of its particles' factors.
// The footprint bounds use the reference's FP64 truncation; kernel values and
// the per-pixel walk are FP32 (one absorbed fraction 1 - exp(-tau) per band
// and particle, I <- I + (1 - exp(-tau)) (S - I)).
#include <cfloat>

#include "mg_common.cuh"
#include "mg_scan.cuh"

namespace mg {

constexpr int kRtTile = 32;      // pixels per tile side
constexpr int kRtThreads = 256;  // 4 pixels per thread
constexpr int kRtChunk = 1024;   // particles per work item
constexpr int kRtBatch = 128;    // particles staged in shared memory at a time
constexpr int kRtMaxBands = 8;
constexpr float kKernel2dNorm = 1.8189136353359467f;  // 40 / (7 pi) (kernel2d)

// Footprint of particle i in pixels, as the reference computes it (h at least
// dx, C truncation, clipped to the grid).  Returns false when it deposits
// nothing (h == 0, m == 0, or no pixel).
__device__ __forceinline__ bool rt_footprint(const double *__restrict__ x, const double *__restrict__ h,
                                             const double *__restrict__ m, int64_t i, double L, double cx, double cy,
                                             double dx, int res, double &xs0, double &xs1, double &hs, int g[4]) {
    xs0 = x[i * 3 + 0] - cx + L / 2;
    xs1 = x[i * 3 + 1] - cy + L / 2;
    hs = fmax(h[i], dx);
    if (hs == 0 || m[i] == 0) return false;
    g[0] = max((int)((xs0 - hs) / dx + 1), 0);
    g[1] = min((int)((xs0 + hs) / dx), res - 1);
    g[2] = max((int)((xs1 - hs) / dx + 1), 0);
    g[3] = min((int)((xs1 + hs) / dx), res - 1);
    return g[1] >= g[0] && g[3] >= g[2];
}

// Order-preserving u64 of a double, complemented so that ascending keys are
// descending values.
__device__ __forceinline__ uint64_t rt_desc_key(double v) {
    const uint64_t b = (uint64_t)__double_as_longlong(v);
    const uint64_t o = (b >> 63) ? ~b : (b | 0x8000000000000000ull);
    return ~o;
}

__global__ void k_rt_keys(const double *__restrict__ x, int64_t n, double cz, uint64_t *__restrict__ keys,
                          int32_t *__restrict__ vals) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    keys[i] = rt_desc_key(x[i * 3 + 2] - cz);
    vals[i] = (int32_t)i;
}

// pairs per particle (in z order when order != null), and their total
__global__ void k_rt_count(const double *__restrict__ x, const double *__restrict__ h, const double *__restrict__ m,
                           const int32_t *__restrict__ order, int64_t n, double L, double cx, double cy, int res,
                           uint32_t *__restrict__ pcount, unsigned long long *__restrict__ total) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    uint32_t c = 0;
    if (r < n) {
        const int64_t i = order ? order[r] : r;
        const double dx = L / (double)(res - 1);
        double xs0, xs1, hs;
        int g[4];
        if (rt_footprint(x, h, m, i, L, cx, cy, dx, res, xs0, xs1, hs, g))
            c = (uint32_t)((g[1] / kRtTile - g[0] / kRtTile + 1) * (g[3] / kRtTile - g[2] / kRtTile + 1));
        if (pcount) pcount[r] = c;
    }
    if (total) {
        const unsigned long long s = warp_sum((unsigned long long)c);
        if ((threadIdx.x & 31) == 0 && s) atomicAdd(total, s);
    }
}

__global__ void k_rt_pairs(const double *__restrict__ x, const double *__restrict__ h, const double *__restrict__ m,
                           const int32_t *__restrict__ order, int64_t n, double L, double cx, double cy, int res,
                           const uint32_t *__restrict__ poff, uint64_t *__restrict__ pkey,
                           int32_t *__restrict__ pval) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int64_t i = order[r];
    const double dx = L / (double)(res - 1);
    double xs0, xs1, hs;
    int g[4];
    if (!rt_footprint(x, h, m, i, L, cx, cy, dx, res, xs0, xs1, hs, g)) return;
    const int ntx = (res + kRtTile - 1) / kRtTile;
    int64_t e = poff[r];
    for (int tx = g[0] / kRtTile; tx <= g[1] / kRtTile; ++tx)
        for (int ty = g[2] / kRtTile; ty <= g[3] / kRtTile; ++ty, ++e) {
            pkey[e] = ((uint64_t)(tx * ntx + ty) << 32) | (uint64_t)r;
            pval[e] = (int32_t)i;
        }
}

// tile t's pairs are [tbeg[t], tbeg[t + 1]) of the tile-sorted pairs
__global__ void k_rt_tile_starts(const uint64_t *__restrict__ pkey, int64_t npairs, int ntiles,
                                 uint32_t *__restrict__ tbeg) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e > npairs) return;
    const int t = e < npairs ? (int)(pkey[e] >> 32) : ntiles;
    const int tp = e > 0 ? (int)(pkey[e - 1] >> 32) : -1;
    for (int u = tp + 1; u <= t; ++u) tbeg[u] = (uint32_t)e;
}

__global__ void k_rt_item_count(const uint32_t *__restrict__ tbeg, int ntiles, uint32_t *__restrict__ icount) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < ntiles) icount[t] = (tbeg[t + 1] - tbeg[t] + kRtChunk - 1) / kRtChunk;
    if (t == ntiles) icount[t] = 0;
}

__global__ void k_rt_items(const uint32_t *__restrict__ tbeg, const uint32_t *__restrict__ ioff, int ntiles,
                           int4 *__restrict__ items) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntiles) return;
    const uint32_t b = tbeg[t], e = tbeg[t + 1];
    uint32_t it = ioff[t];
    for (uint32_t s = b; s < e; s += kRtChunk, ++it) items[it] = make_int4(t, (int)s, (int)min(e, s + kRtChunk), 0);
}

// 1 - exp(-t), the fraction of the light a layer of optical depth t absorbs
// (-expm1(-t)).  Below t = 1/8 from its Taylor series to degree 6,
// t (1 - t/2 (1 - t/3 (1 - t/4 (1 - t/5 (1 - t/6))))), whose truncation is
// below t^6 / 5040 < 8e-10 of the value there; above, the library's expm1f.
// The exchange step I <- exp(-t) I + (1 - exp(-t)) S is then I + p (S - I):
// one factor instead of an exponential and an expm1 per pixel, particle and
// band (the ray tracer's inner loop is bound by instruction issue).
__device__ __forceinline__ float absorbed(float t) {
    if (fabsf(t) < 0.125f) {
        float q = fmaf(-t, 1.0f / 6.0f, 1.0f);
        q = fmaf(-t * 0.2f, q, 1.0f);
        q = fmaf(-t * 0.25f, q, 1.0f);
        q = fmaf(-t * (1.0f / 3.0f), q, 1.0f);
        q = fmaf(-t * 0.5f, q, 1.0f);
        return t * q;
    }
    return -expm1f(-t);
}

struct RtParticle {
    float fx, fy, hpx2_inv, mh2;  // position / dx, 1 / (h / dx)^2, m / h^2
    int g[4];                     // clipped footprint bounds
};

template <int B>
__global__ __launch_bounds__(kRtThreads) void k_rt_chunk(const int4 *__restrict__ items,
                                                        const uint32_t *__restrict__ nitems,
                                                        const int32_t *__restrict__ pval, const double *__restrict__ x,
                                                        const double *__restrict__ h, const double *__restrict__ m,
                                                        const double *__restrict__ kappa,
                                                        const double *__restrict__ j, double L, double cx, double cy,
                                                        int res, float *__restrict__ ci, float *__restrict__ ct) {
    __shared__ RtParticle sp[kRtBatch];
    __shared__ float skap[kRtBatch][B], ssrc[kRtBatch][B];
    const int item = blockIdx.x;
    if (item >= (int)*nitems) return;
    const int4 it = items[item];
    const int ntx = (res + kRtTile - 1) / kRtTile;
    const int tx = it.x / ntx, ty = it.x % ntx;
    const int tid = threadIdx.x;
    const int gx = tx * kRtTile + (tid & 31);
    int gy[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) gy[k] = ty * kRtTile + (tid >> 5) + 8 * k;
    float I[4][B], T[4][B];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int b = 0; b < B; ++b) I[k][b] = T[k][b] = 0.0f;
    const double dx = L / (double)(res - 1);
    for (int s0 = it.y; s0 < it.z; s0 += kRtBatch) {
        const int nb = min(kRtBatch, it.z - s0);
        __syncthreads();
        if (tid < nb) {
            const int64_t i = pval[s0 + tid];
            double xs0, xs1, hs;
            RtParticle q;
            rt_footprint(x, h, m, i, L, cx, cy, dx, res, xs0, xs1, hs, q.g);
            q.fx = (float)(xs0 / dx);
            q.fy = (float)(xs1 / dx);
            const float hp = (float)(hs / dx);
            q.hpx2_inv = 1.0f / (hp * hp);
            q.mh2 = (float)(m[i] / (hs * hs));
            sp[tid] = q;
#pragma unroll
            for (int b = 0; b < B; ++b) {
                const float kp = (float)kappa[i * B + b];
                skap[tid][b] = kp;
                ssrc[tid][b] = kp > 0.0f ? (float)(j[i * B + b] / (4.0 * 3.14159265358979323846 * kappa[i * B + b] + 1e-100))
                                         : 0.0f;
            }
        }
        __syncthreads();
        for (int p = 0; p < nb; ++p) {
            const RtParticle q = sp[p];
            if (gx < q.g[0] || gx > q.g[1]) continue;
            const float ddx = (float)gx - q.fx;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (gy[k] < q.g[2] || gy[k] > q.g[3]) continue;
                const float ddy = (float)gy[k] - q.fy;
                const float q2 = fmaf(ddy, ddy, ddx * ddx) * q.hpx2_inv;
                if (q2 > 1.0f) continue;
                // |d| / h as q2 rsqrt(q2) (q2 <= 1 here); the kernel value
                // times m / h^2 once for all bands
                const float kmh = kKernel2dNorm * spline_w(q2 * rsqrtf(fmaxf(q2, 1e-30f))) * q.mh2;
#pragma unroll
                for (int b = 0; b < B; ++b) {
                    const float tau = skap[p][b] * kmh;
                    T[k][b] += tau;
                    I[k][b] = fmaf(absorbed(tau), ssrc[p][b] - I[k][b], I[k][b]);
                }
            }
        }
    }
    // chunk result for the tile's pixels: [item][pixel in tile][band]
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int lp = (tid & 31) * kRtTile + (tid >> 5) + 8 * k;
#pragma unroll
        for (int b = 0; b < B; ++b) {
            ci[((int64_t)item * kRtTile * kRtTile + lp) * B + b] = I[k][b];
            ct[((int64_t)item * kRtTile * kRtTile + lp) * B + b] = T[k][b];
        }
    }
}

// Front-to-back composition of each pixel's chunks (the last chunk of a tile
// holds its nearest particles) plus the attenuated background.
__global__ void k_rt_combine(const uint32_t *__restrict__ ioff, const float *__restrict__ ci,
                             const float *__restrict__ ct, const double *__restrict__ i0, int res, int B,
                             double *__restrict__ inten, double *__restrict__ taumap) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= (int64_t)res * res) return;
    const int gx = (int)(c / res), gy = (int)(c % res);
    const int ntx = (res + kRtTile - 1) / kRtTile;
    const int t = (gx / kRtTile) * ntx + gy / kRtTile;
    const int lp = (gx % kRtTile) * kRtTile + gy % kRtTile;
    const int i0_ = (int)ioff[t], i1 = (int)ioff[t + 1];
    for (int b = 0; b < B; ++b) {
        double acc = 0.0, tau = 0.0;
        for (int it = i1 - 1; it >= i0_; --it) {
            const int64_t o = ((int64_t)it * kRtTile * kRtTile + lp) * B + b;
            acc += (double)ci[o] * exp(-tau);
            tau += (double)ct[o];
        }
        if (i0) acc += i0[b] * exp(-tau);
        inten[c * B + b] = acc;
        if (taumap) taumap[c * B + b] = tau;
    }
}

template <int B>
static void launch_rt_chunk(unsigned grid, cudaStream_t st, const int4 *items, const uint32_t *nitems,
                            const int32_t *pval, const double *x, const double *h, const double *m,
                            const double *kappa, const double *j, double L, double cx, double cy, int res, float *ci,
                            float *ct) {
    k_rt_chunk<B><<<grid, kRtThreads, 0, st>>>(items, nitems, pval, x, h, m, kappa, j, L, cx, cy, res, ci, ct);
}

struct RtLayout {
    int ntiles;
    int64_t max_items;
};

static RtLayout rt_layout(int64_t npairs, int res) {
    RtLayout l;
    const int ntx = (res + kRtTile - 1) / kRtTile;
    l.ntiles = ntx * ntx;
    l.max_items = (int64_t)l.ntiles + npairs / kRtChunk + 1;
    return l;
}

}  // namespace mg

using namespace mg;

extern "C" int mg_radtransfer_count(const double *pos, const double *h, const double *m, int64_t n, int32_t res,
                                    double L, double cx, double cy, int64_t *npairs, void *stream_) {
    if (!npairs || n < 0 || res < 2 || !(L > 0.0) || (n > 0 && (!pos || !h || !m))) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    MG_CUDA(cudaMemsetAsync(npairs, 0, sizeof(int64_t), st));
    if (n == 0) return MG_OK;
    k_rt_count<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(pos, h, m, nullptr, n, L, cx, cy, res, nullptr,
                                                            reinterpret_cast<unsigned long long *>(npairs));
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" size_t mg_radtransfer_workspace_bytes(int64_t n, int64_t npairs, int32_t res, int32_t bands) {
    if (n < 0 || npairs < 0 || res < 2 || bands < 1) return 0;
    const RtLayout l = rt_layout(npairs, res);
    const int64_t m = n > npairs ? n : npairs;
    return align_up(sizeof(uint64_t) * (size_t)(n + 1)) + 2 * align_up(sizeof(int32_t) * (size_t)(m + 1)) +
           align_up(sizeof(uint32_t) * (size_t)(n + 1)) + align_up(scan_workspace_bytes(n + 1)) +
           align_up(sizeof(uint64_t) * (size_t)(npairs + 1)) + radix_sort_workspace_bytes(m + 1) +
           3 * align_up(sizeof(uint32_t) * (size_t)(l.ntiles + 2)) + align_up(scan_workspace_bytes(l.ntiles + 1)) +
           align_up(sizeof(int4) * (size_t)l.max_items) +
           2 * align_up(sizeof(float) * (size_t)l.max_items * kRtTile * kRtTile * (size_t)bands) + 4096;
}

extern "C" int mg_radtransfer(const double *j, const double *m, const double *kappa, const double *pos,
                              const double *h, int64_t n, int32_t bands, int32_t res, double L, double cx, double cy,
                              double cz, const double *i0, int64_t npairs, double *intensity, double *tau,
                              void *workspace, size_t workspace_bytes, void *stream_) {
    if (!intensity || n < 0 || res < 2 || !(L > 0.0) || (n > 0 && (!j || !m || !kappa || !pos || !h)))
        return MG_ERR_ARG;
    if (bands < 1 || bands > kRtMaxBands) return MG_ERR_UNSUPPORTED;
    if (npairs < 0 || npairs > 0x7fffffffll || n > 0x7fffffffll) return MG_ERR_UNSUPPORTED;
    if (workspace_bytes < mg_radtransfer_workspace_bytes(n, npairs, res, bands)) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    const RtLayout l = rt_layout(npairs, res);
    const int64_t mm = n > npairs ? n : npairs;
    Carve w(workspace, workspace_bytes);
    uint64_t *zkey = w.take<uint64_t>((size_t)n + 1);
    int32_t *order = w.take<int32_t>((size_t)mm + 1);
    int32_t *pval = w.take<int32_t>((size_t)mm + 1);
    uint32_t *pcount = w.take<uint32_t>((size_t)n + 1);
    void *scan_ws = w.take<char>(scan_workspace_bytes(n + 1));
    uint64_t *pkey = w.take<uint64_t>((size_t)npairs + 1);
    void *sort_ws = w.take<char>(radix_sort_workspace_bytes(mm + 1));
    uint32_t *tbeg = w.take<uint32_t>((size_t)l.ntiles + 2);
    uint32_t *ioff = w.take<uint32_t>((size_t)l.ntiles + 2);
    uint32_t *nitems = w.take<uint32_t>((size_t)l.ntiles + 2);
    void *scan_ws2 = w.take<char>(scan_workspace_bytes(l.ntiles + 1));
    int4 *items = w.take<int4>((size_t)l.max_items);
    float *ci = w.take<float>((size_t)l.max_items * kRtTile * kRtTile * (size_t)bands);
    float *ct = w.take<float>((size_t)l.max_items * kRtTile * kRtTile * (size_t)bands);
    if (!w.ok()) return MG_ERR_ARG;
    const unsigned gb = (unsigned)((n + 255) / 256);
    // 1. particles by z, descending (stable: ties by index)
    if (n > 0) {
        k_rt_keys<<<gb, 256, 0, st>>>(pos, n, cz, zkey, order);
        MG_CHECK_LAUNCH();
        int rc = radix_sort_pairs(zkey, order, n, 0, 64, sort_ws, radix_sort_workspace_bytes(mm + 1), st);
        if (rc) return rc;
        // 2. (tile, rank) pairs in z order, stably sorted by tile
        k_rt_count<<<gb, 256, 0, st>>>(pos, h, m, order, n, L, cx, cy, res, pcount, nullptr);
        MG_CHECK_LAUNCH();
        MG_CUDA(cudaMemsetAsync(pcount + n, 0, sizeof(uint32_t), st));
        rc = exclusive_scan_u32(pcount, pcount, n + 1, scan_ws, st);
        if (rc) return rc;
        k_rt_pairs<<<gb, 256, 0, st>>>(pos, h, m, order, n, L, cx, cy, res, pcount, pkey, pval);
        MG_CHECK_LAUNCH();
    }
    int tile_bits = 1;
    while ((1 << tile_bits) < l.ntiles) ++tile_bits;
    if (npairs > 1) {
        int rc = radix_sort_pairs(pkey, pval, npairs, 32, tile_bits, sort_ws, radix_sort_workspace_bytes(mm + 1), st);
        if (rc) return rc;
    }
    // 3. tiles -> chunks of kRtChunk pairs
    MG_CUDA(cudaMemsetAsync(tbeg, 0, sizeof(uint32_t) * ((size_t)l.ntiles + 1), st));
    k_rt_tile_starts<<<(unsigned)((npairs + 1 + 255) / 256), 256, 0, st>>>(pkey, npairs, l.ntiles, tbeg);
    MG_CHECK_LAUNCH();
    k_rt_item_count<<<(unsigned)((l.ntiles + 1 + 255) / 256), 256, 0, st>>>(tbeg, l.ntiles, ioff);
    MG_CHECK_LAUNCH();
    int rc = exclusive_scan_u32(ioff, ioff, l.ntiles + 1, scan_ws2, st);
    if (rc) return rc;
    MG_CUDA(cudaMemcpyAsync(nitems, ioff + l.ntiles, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    k_rt_items<<<(unsigned)((l.ntiles + 255) / 256), 256, 0, st>>>(tbeg, ioff, l.ntiles, items);
    MG_CHECK_LAUNCH();
    // 4. walk each chunk, then compose the chunks per pixel
    if (l.max_items > 0) {
        const unsigned grid = (unsigned)l.max_items;
        switch (bands) {
            case 1: launch_rt_chunk<1>(grid, st, items, nitems, pval, pos, h, m, kappa, j, L, cx, cy, res, ci, ct); break;
            case 2: launch_rt_chunk<2>(grid, st, items, nitems, pval, pos, h, m, kappa, j, L, cx, cy, res, ci, ct); break;
            case 3: launch_rt_chunk<3>(grid, st, items, nitems, pval, pos, h, m, kappa, j, L, cx, cy, res, ci, ct); break;
            case 4: launch_rt_chunk<4>(grid, st, items, nitems, pval, pos, h, m, kappa, j, L, cx, cy, res, ci, ct); break;
            case 5: launch_rt_chunk<5>(grid, st, items, nitems, pval, pos, h, m, kappa, j, L, cx, cy, res, ci, ct); break;
            case 6: launch_rt_chunk<6>(grid, st, items, nitems, pval, pos, h, m, kappa, j, L, cx, cy, res, ci, ct); break;
            case 7: launch_rt_chunk<7>(grid, st, items, nitems, pval, pos, h, m, kappa, j, L, cx, cy, res, ci, ct); break;
            default: launch_rt_chunk<8>(grid, st, items, nitems, pval, pos, h, m, kappa, j, L, cx, cy, res, ci, ct); break;
        }
        MG_CHECK_LAUNCH();
    }
    const int64_t cells = (int64_t)res * res;
    k_rt_combine<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(ioff, ci, ct, i0, res, bands, intensity, tau);
    MG_CHECK_LAUNCH();
    return MG_OK;
}
