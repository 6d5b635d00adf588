// Projected maps and point queries:
//  * mg_surface_density: column-integrated cubic-spline deposition
//    (src/meshoid/grid_deposition.py:123-295), tile-binned: particles whose
//    footprint spans at most 2x2 tiles of 32x32 pixels are binned to tiles with
//    a counting sort (per-tile counters, scan, scatter) and each tile is
//    accumulated in shared memory by one CTA and written once -- no global
//    atomics.  Particles with larger footprints are listed; one CTA per tile
//    streams that list through shared memory in chunks, keeps the particles
//    whose footprint meets the tile and sums their contributions to its
//    pixels in registers (no atomics) -- when their footprints cover a good
//    share of the map; otherwise a per-particle CTA adds into the grid with
//    FP64 atomics.
//  * mg_nn_query: nearest particle of arbitrary points, the k = 1 query behind
//    Reconstruct / Slice (src/meshoid/Meshoid.py:407-411).
#include <algorithm>
#include <cfloat>

#include "mg_common.cuh"
#include "mg_maps.cuh"
#include "mg_scan.cuh"

namespace mg {

constexpr int kTile = 32;
constexpr float kKernel2dNorm = 1.8189136353359467f;  // 40 / (7 pi), grid_deposition.py kernel2d

struct SdParticle {
    float rx, ry;   // position relative to pixel node (gx0, gy0), FP32
    float h;        // smoothing length (conservative: max(h, dx))
    float coef;     // f / h^2 (standard) or f / total_weight (conservative)
    int gx0, gx1, gy0, gy1;
};

struct SdArgs {
    const double *pos;
    const double *h;
    const double *f;
    int64_t n;
    double cx, cy, size, dx, inv_dx;
    int res, conservative, ntx;
    SdParticle *rec;
    uint32_t *tile_count;  // ntiles + 1
    uint32_t *ranks;       // 4 per particle
    int32_t *big_list;
    uint32_t *big_count;
    int32_t *pairs;
    uint32_t *item_off;  // ntiles + 1: first work item of each tile (tiles split into chunks of kSdChunk pairs)
    double *grid;
    // large footprints binned per tile: (tile, particle) pairs
    uint32_t *btile;      // ntiles + 1: pairs per tile, then their offsets
    uint32_t *bfill;      // ntiles: scatter cursors
    int32_t *bpairs;      // bcap: particle of each pair, grouped by tile
    uint32_t *bitem_off;  // ntiles + 1: first work item of each tile (chunks of kSdBigChunk pairs)
    uint64_t bcap;
};

constexpr int kSdChunk = 2048;     // pairs per work item of k_sd_tile
constexpr int kSdBigChunk = 1024;  // pairs per work item of k_sd_tile_pairs

// Footprint of particle i exactly as the reference computes it (FP64, C
// truncation toward zero), grid_deposition.py:200-216 / :248-265.
// v / dx as the reference divides it (FP64, round to nearest): v * (1/dx) is
// within 2 ulp of it, which can change the truncation that follows only
// when the quotient lies that close to an integer; only then is the
// division done (FP64 division is slow on this GPU).
__device__ __forceinline__ double sd_div(double v, const SdArgs &a) {
    const double y = v * a.inv_dx;
    const double r = rint(y);
    return fabs(y - r) <= 1e-12 * fabs(y) + 1e-300 ? v / a.dx : y;
}

// The two truncations of one axis in FP32: y0 = (x - h) / dx + 1 and
// y1 = (x + h) / dx from the FP32 roundings of x and h, each within
// ~4e-7 (|x| + h) / dx of the FP64 values the reference truncates.  Where
// either lies within 1e-6 (|x| + h) / dx + 1e-6 of an integer (~0.1% of
// them) the caller decides in FP64 instead.
__device__ __forceinline__ bool sd_bounds32(float x, float h, float inv_dx, int res, int &g0, int &g1) {
    int a, b;
    if (!trunc_pair32(x, h, inv_dx, a, b)) return false;
    g0 = max(a, 0);
    g1 = min(b, res - 1);
    return true;
}

__device__ __forceinline__ bool footprint(const SdArgs &a, int64_t i, double &xs0, double &xs1, double &hs,
                                          int &gx0, int &gx1, int &gy0, int &gy1) {
    xs0 = a.pos[i * 3 + 0] - a.cx + a.size * 0.5;
    xs1 = a.pos[i * 3 + 1] - a.cy + a.size * 0.5;
    hs = a.h[i];
    if (a.conservative && hs < a.dx) hs = a.dx;
    // FP32 decides the truncations wherever it can tell (conversions and
    // divisions in FP64 run at a small fraction of the FP32 rate here)
    const float hf = (float)hs, invf = (float)a.inv_dx;
    const bool fx = sd_bounds32((float)xs0, hf, invf, a.res, gx0, gx1);
    const bool fy = sd_bounds32((float)xs1, hf, invf, a.res, gy0, gy1);
    if (!fx) {
        gx0 = max((int)(sd_div(xs0 - hs, a) + 1.0), 0);
        gx1 = min((int)sd_div(xs0 + hs, a), a.res - 1);
    }
    if (!fy) {
        gy0 = max((int)(sd_div(xs1 - hs, a) + 1.0), 0);
        gy1 = min((int)sd_div(xs1 + hs, a), a.res - 1);
    }
    return gx0 <= gx1 && gy0 <= gy1;
}

constexpr int kSdPrepTiles = 4096;  // tile counters a block of k_sd_prep sums in shared memory first

__global__ __launch_bounds__(256) void k_sd_prep(SdArgs a) {
    __shared__ uint32_t sh_tile[kSdPrepTiles];
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int ntiles = a.ntx * a.ntx;
    const bool blocksum = ntiles <= kSdPrepTiles;  // the same in every block
    if (blocksum) {
        for (int t = threadIdx.x; t < ntiles; t += blockDim.x) sh_tile[t] = 0u;
        __syncthreads();
    }
    double xs0 = 0, xs1 = 0, hs = 1;
    int gx0 = 0, gx1 = -1, gy0 = 0, gy1 = -1;
    bool any = false;
    if (i < a.n) any = footprint(a, i, xs0, xs1, hs, gx0, gx1, gy0, gy1);
    int tx0 = gx0 / kTile, tx1 = gx1 / kTile, ty0 = gy0 / kTile, ty1 = gy1 / kTile;
    const bool big = any && (tx1 - tx0 > 1 || ty1 - ty0 > 1);
    const bool small = any && !big;
    if (i < a.n) {
        SdParticle r;
        r.rx = (float)(xs0 - gx0 * a.dx);
        r.ry = (float)(xs1 - gy0 * a.dx);
        r.h = (float)hs;
        // stored in FP32: formed in FP32 (a few ulp; an FP64 division per
        // particle was a large share of this pass on this GPU), in FP64 only
        // where FP32 over- or underflows
        const float hf = (float)hs, hh = hf * hf;
        float c = hh > 0.0f ? (float)a.f[i] / hh : 0.0f;
        if (!(hh > 0.0f) || !isfinite(c)) c = (float)(a.f[i] / (hs * hs));
        r.coef = any && !a.conservative ? c : 0.0f;
        r.gx0 = gx0; r.gx1 = gx1; r.gy0 = gy0; r.gy1 = gy1;
        if (any && a.conservative && !big) {
            // total kernel weight over the whole footprint (normalisation; a
            // large footprint's is summed by a warp in k_sd_cons_norm)
            const float hf = (float)hs, hinv = 1.0f / hf, dxf = (float)a.dx;
            float tot = 0.0f, comp = 0.0f;
            for (int gx = gx0; gx <= gx1; ++gx) {
                const float ddx = r.rx - (float)(gx - gx0) * dxf;
                for (int gy = gy0; gy <= gy1; ++gy) {
                    const float ddy = r.ry - (float)(gy - gy0) * dxf;
                    const float rr = sqrtf(ddx * ddx + ddy * ddy);
                    if (rr > hf) continue;
                    const float y = spline_w(rr * hinv) * kKernel2dNorm - comp;
                    const float t = tot + y;
                    comp = (t - tot) - y;
                    tot = t;
                }
            }
            r.coef = tot > 0.0f ? (float)(a.f[i] / (double)tot) : 0.0f;
            if (!(tot > 0.0f)) r.gx1 = r.gx0 - 1;  // nothing to deposit
        }
        a.rec[i] = r;
    }
    // small particles: one counter increment per overlapped tile (<= 4).
    // Particles come in input order, so a warp's tiles rarely agree and the
    // counters of a dense core's few tiles took ~10^5 global atomics each:
    // a block sums its increments in shared memory and adds one per tile.
    if (blocksum) {
        uint32_t loc[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int tx = tx0 + (u & 1), ty = ty0 + (u >> 1);
            const bool valid = small && tx <= tx1 && ty <= ty1;
            loc[u] = valid ? atomicAdd(&sh_tile[tx * a.ntx + ty], 1u) : 0xffffffffu;
        }
        __syncthreads();
        for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
            const uint32_t c = sh_tile[t];
            if (c) sh_tile[t] = atomicAdd(&a.tile_count[t], c);  // the block's base in tile t
        }
        __syncthreads();
        if (i < a.n) {
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int tx = tx0 + (u & 1), ty = ty0 + (u >> 1);
                a.ranks[i * 4 + u] = loc[u] != 0xffffffffu ? sh_tile[tx * a.ntx + ty] + loc[u] : 0xffffffffu;
            }
        }
    }
    // otherwise aggregated across the warp for equal tiles
    for (int u = 0; u < 4 && !blocksum; ++u) {
        const int tx = tx0 + (u & 1), ty = ty0 + (u >> 1);
        const bool valid = small && tx <= tx1 && ty <= ty1;
        const uint32_t t = valid ? (uint32_t)(tx * a.ntx + ty) : 0xffffffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, t);
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (valid && lane == leader) base = atomicAdd(&a.tile_count[t], (uint32_t)__popc(peers));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (i < a.n) a.ranks[i * 4 + u] = valid ? base + __popc(peers & ((1u << lane) - 1u)) : 0xffffffffu;
    }
    // large footprints: list slots and footprint pixels, one atomic per warp
    // for each (a particle's own atomics on these two words serialised the
    // pass: ~18% of a Plummer sphere's particles are large at 1024^2)
    const unsigned bm = __ballot_sync(0xffffffffu, big);
    if (bm) {
        const int leader = __ffs(bm) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(a.big_count, (uint32_t)__popc(bm));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (big) a.big_list[base + __popc(bm & ((1u << lane) - 1u))] = (int32_t)i;
        unsigned long long px = big ? (unsigned long long)(gx1 - gx0 + 1) * (unsigned long long)(gy1 - gy0 + 1) : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) px += __shfl_xor_sync(0xffffffffu, px, o);
        if (lane == leader) atomicAdd(reinterpret_cast<unsigned long long *>(a.big_count + 2), px);  // footprint pixels
    }
}

// Conservative deposit, large footprints: the total kernel weight over the
// footprint (the normalisation), one warp per listed particle, lanes over its
// pixels (Kahan sums per lane, combined in FP64); one thread per particle
// would walk up to res^2 pixels alone.  Sets the coefficient, or empties the
// footprint when the total is zero, before the pairs are counted.
__global__ __launch_bounds__(256) void k_sd_cons_norm(SdArgs a) {
    const uint32_t nb = a.big_count[0];
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float dxf = (float)a.dx;
    for (int64_t b = warp; b < (int64_t)nb; b += nwarps) {
        const int32_t i = a.big_list[b];
        const SdParticle r = a.rec[i];
        const int hgt = r.gy1 - r.gy0 + 1;
        const int64_t npx = (int64_t)(r.gx1 - r.gx0 + 1) * hgt;
        const float hinv = 1.0f / r.h;
        float tot = 0.0f, comp = 0.0f;
        for (int64_t t = lane; t < npx; t += 32) {
            const int gx = r.gx0 + (int)(t / hgt), gy = r.gy0 + (int)(t % hgt);
            const float ddx = r.rx - (float)(gx - r.gx0) * dxf;
            const float ddy = r.ry - (float)(gy - r.gy0) * dxf;
            const float rr = sqrtf(ddx * ddx + ddy * ddy);
            if (rr > r.h) continue;
            const float y = spline_w(rr * hinv) * kKernel2dNorm - comp;
            const float u = tot + y;
            comp = (u - tot) - y;
            tot = u;
        }
        double sum = (double)tot - (double)comp;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        if (lane == 0) {
            a.rec[i].coef = sum > 0.0 ? (float)(a.f[i] / sum) : 0.0f;
            if (!(sum > 0.0)) a.rec[i].gx1 = r.gx0 - 1;  // nothing to deposit
        }
    }
}

__global__ void k_sd_scatter(SdArgs a) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const SdParticle r = a.rec[i];
    const int tx0 = r.gx0 / kTile, ty0 = r.gy0 / kTile;
    for (int u = 0; u < 4; ++u) {
        const uint32_t rk = a.ranks[i * 4 + u];
        if (rk == 0xffffffffu) continue;
        const int tx = tx0 + (u & 1), ty = ty0 + (u >> 1);
        a.pairs[a.tile_count[tx * a.ntx + ty] + rk] = (int32_t)i;
    }
}

// Work items per tile: ceil(pairs / kSdChunk), at least 1 (an empty tile still
// writes its zeros).
__global__ void k_sd_items(SdArgs a, int64_t ntiles) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < ntiles) {
        const uint32_t c = a.tile_count[t + 1] - a.tile_count[t];
        a.item_off[t] = c <= (uint32_t)kSdChunk ? 1u : (c + kSdChunk - 1) / kSdChunk;
    } else if (t == ntiles) {
        a.item_off[t] = 0u;
    }
}

// One CTA per work item (a tile, or a chunk of kSdChunk pairs of a crowded
// tile): shared-memory accumulation; a tile of one item stores its pixels, the
// chunks of a split tile add theirs atomically into the zeroed grid.
__global__ __launch_bounds__(256) void k_sd_tile(SdArgs a, int64_t ntiles) {
    __shared__ float acc[kTile][kTile + 1];
    const uint32_t item = blockIdx.x;
    if (item >= a.item_off[ntiles]) return;
    int64_t lo = 0, hi = ntiles - 1;  // tile: largest t with item_off[t] <= item
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (a.item_off[mid] <= item)
            lo = mid;
        else
            hi = mid - 1;
    }
    const int tile = (int)lo;
    const uint32_t nitems = a.item_off[tile + 1] - a.item_off[tile];
    const uint32_t j = item - a.item_off[tile];
    const int tx = tile / a.ntx, ty = tile % a.ntx;
    for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) acc[e / kTile][e % kTile] = 0.0f;
    __syncthreads();
    const uint32_t t0 = a.tile_count[tile], t1 = a.tile_count[tile + 1];
    const uint32_t b0 = t0 + j * (uint32_t)kSdChunk, b1 = min(t1, b0 + (uint32_t)kSdChunk);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const float dxf = (float)a.dx;
    const int px0 = tx * kTile, py0 = ty * kTile;
    for (uint32_t e = b0 + warp; e < b1; e += nwarp) {
        const SdParticle r = a.rec[a.pairs[e]];
        const int x0 = max(r.gx0, px0), x1 = min(r.gx1, px0 + kTile - 1);
        const int y0 = max(r.gy0, py0), y1 = min(r.gy1, py0 + kTile - 1);
        const int w = x1 - x0 + 1, hgt = y1 - y0 + 1;
        if (w <= 0 || hgt <= 0) continue;
        const float hinv = 1.0f / r.h;
        const float coef2 = 2.0f * (r.coef * kKernel2dNorm);
        // pixel t of the footprint's part of the tile (w x hgt <= 32 x 32):
        // row t / hgt by an FP32 reciprocal, exact for t < 2^10 ((t + 1/2) /
        // hgt is at least 1/(2 hgt) from an integer); offsets from the
        // footprint's first node as exact small floats; |d| by r^2 rsqrt(r^2)
        const float h2 = r.h * r.h, hf = (float)hgt, inv = 1.0f / hf;
        const float fx0 = (float)(x0 - r.gx0), fy0 = (float)(y0 - r.gy0);
        float *accf = &acc[0][0] + (x0 - px0) * (kTile + 1) + (y0 - py0);
        const int skew = kTile + 1 - hgt;
        for (int t = lane; t < w * hgt; t += 32) {
            const float tf = (float)t;
            const float rf = floorf((tf + 0.5f) * inv);
            const float cf = fmaf(-rf, hf, tf);
            const float ddx = fmaf(-(fx0 + rf), dxf, r.rx);
            const float ddy = fmaf(-(fy0 + cf), dxf, r.ry);
            const float r2 = fmaf(ddx, ddx, ddy * ddy);
            if (r2 > h2) continue;
            atomicAdd(accf + t + (int)rf * skew, spline_w_half(r2 * rsqrtf(fmaxf(r2, 1e-30f)) * hinv) * coef2);
        }
    }
    __syncthreads();
    const double scale = a.conservative ? 1.0 / (a.dx * a.dx) : 1.0;
    for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
        const int gx = px0 + e / kTile, gy = py0 + e % kTile;
        if (gx >= a.res || gy >= a.res) continue;
        const double v = (double)acc[e / kTile][e % kTile] * scale;
        if (nitems == 1)
            a.grid[(int64_t)gx * a.res + gy] = v;
        else if (v != 0.0)
            atomicAdd(&a.grid[(int64_t)gx * a.res + gy], v);
    }
}

// Large footprints, gathered per tile: the listed particles are streamed in
// chunks of 256 records; those whose footprint meets this tile are compacted
// in shared memory and every thread adds their contributions to its 4 pixels
// (pixel e = threadIdx.x + 256 j of the tile) in registers.  Runs after
// k_sd_tile, which wrote the tile's pixels, and adds to them.
constexpr int64_t kSdGatherLimit = int64_t(1) << 28;  // listed particles x tiles scanned at most

// The gather scans every listed particle for every tile (~9 ps per check on
// a GB300) and then evaluates whole tiles in registers (~2 ps per pixel); the
// FP64-atomic path costs ~5 ps per footprint pixel.  So the gather is taken
// when the footprint pixels are at least 3x (listed particles x tiles).
// big_count[0]: listed particles, big_count[2..3]: their footprint pixels,
// big_count[4..5]: the tiles they cover ((tile, particle) pairs).
__device__ __forceinline__ uint64_t sd_big_pairs(const SdArgs &a) {
    return *reinterpret_cast<const unsigned long long *>(a.big_count + 4);
}
// The per-tile pairs path (k_sd_tile_pairs) is taken whenever the pairs fit
// the buffer; the gather and the FP64-atomic paths remain for the rest.
__device__ __forceinline__ bool sd_pairs(const SdArgs &a) { return sd_big_pairs(a) <= a.bcap; }
__device__ __forceinline__ bool sd_gather(const SdArgs &a) {
    if (sd_pairs(a)) return false;
    const uint64_t nb = a.big_count[0];
    const uint64_t area = *reinterpret_cast<const unsigned long long *>(a.big_count + 2);
    const uint64_t ntiles = (uint64_t)a.ntx * a.ntx;
    return nb > 0 && nb * ntiles <= (uint64_t)kSdGatherLimit && area >= 3 * nb * ntiles;
}

__global__ __launch_bounds__(256) void k_sd_tile_big(SdArgs a) {
    __shared__ SdParticle buf[256];
    __shared__ int wcount[8];
    if (!sd_gather(a)) return;
    const uint32_t nb = *a.big_count;
    const int tile = blockIdx.x;
    const int tx = tile / a.ntx, ty = tile % a.ntx;
    const int px0 = tx * kTile, py0 = ty * kTile;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float dxf = (float)a.dx;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (uint32_t b0 = 0; b0 < nb; b0 += 256) {
        const uint32_t b = b0 + tid;
        SdParticle r;
        bool meets = false;
        if (b < nb) {
            r = a.rec[a.big_list[b]];
            meets = r.coef != 0.0f && r.gx0 <= px0 + kTile - 1 && r.gx1 >= px0 && r.gy0 <= py0 + kTile - 1 &&
                    r.gy1 >= py0;
        }
        const unsigned m = __ballot_sync(0xffffffffu, meets);
        if (lane == 0) wcount[warp] = __popc(m);
        __syncthreads();
        int off = 0, nsel = 0;
        for (int w = 0; w < 8; ++w) {
            off += w < warp ? wcount[w] : 0;
            nsel += wcount[w];
        }
        if (meets) buf[off + __popc(m & ((1u << lane) - 1u))] = r;
        __syncthreads();
        for (int sidx = 0; sidx < nsel; ++sidx) {
            const SdParticle &q = buf[sidx];
            const float hinv = 1.0f / q.h;
            const float coef = q.coef * kKernel2dNorm;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int e = tid + 256 * j;
                const int gx = px0 + e / kTile, gy = py0 + e % kTile;
                if (gx < q.gx0 || gx > q.gx1 || gy < q.gy0 || gy > q.gy1) continue;
                const float ddx = q.rx - (float)(gx - q.gx0) * dxf;
                const float ddy = q.ry - (float)(gy - q.gy0) * dxf;
                const float rr = sqrtf(ddx * ddx + ddy * ddy);
                if (rr > q.h) continue;
                acc[j] += spline_w(rr * hinv) * coef;
            }
        }
        __syncthreads();
    }
    const double scale = a.conservative ? 1.0 / (a.dx * a.dx) : 1.0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int e = tid + 256 * j;
        const int gx = px0 + e / kTile, gy = py0 + e % kTile;
        if (gx < a.res && gy < a.res && acc[j] != 0.0f) a.grid[(int64_t)gx * a.res + gy] += (double)acc[j] * scale;
    }
}

// Large footprints when the per-tile gather would scan too much: one CTA per
// particle, FP64 atomics into the grid.
__global__ __launch_bounds__(256) void k_sd_big(SdArgs a) {
    if (sd_pairs(a) || sd_gather(a)) return;
    const uint32_t nb = *a.big_count;
    const float dxf = (float)a.dx;
    const double scale = a.conservative ? 1.0 / (a.dx * a.dx) : 1.0;
    for (uint32_t b = blockIdx.x; b < nb; b += gridDim.x) {
        const SdParticle r = a.rec[a.big_list[b]];
        const int w = r.gx1 - r.gx0 + 1, hgt = r.gy1 - r.gy0 + 1;
        if (w <= 0 || hgt <= 0) continue;
        const float hinv = 1.0f / r.h;
        const float coef = r.coef * kKernel2dNorm;
        for (int64_t t = threadIdx.x; t < (int64_t)w * hgt; t += blockDim.x) {
            const int gx = r.gx0 + (int)(t / hgt), gy = r.gy0 + (int)(t % hgt);
            const float ddx = r.rx - (float)(gx - r.gx0) * dxf;
            const float ddy = r.ry - (float)(gy - r.gy0) * dxf;
            const float rr = sqrtf(ddx * ddx + ddy * ddy);
            if (rr > r.h) continue;
            atomicAdd(&a.grid[(int64_t)gx * a.res + gy], (double)(spline_w(rr * hinv) * coef) * scale);
        }
    }
}

// Large footprints binned per tile, like the small ones but over every tile a
// footprint covers: one warp per listed particle, lanes over its tiles.
// scatter 0 counts the pairs per tile (and in total); scatter 1, after the
// scan, writes them (only when they fit the buffer).
__global__ __launch_bounds__(256) void k_sd_big_pairs(SdArgs a, int scatter) {
    if (scatter && !sd_pairs(a)) return;
    const uint32_t nb = a.big_count[0];
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long pairs = 0;  // this warp's, added to the total once
    for (int64_t b = warp; b < (int64_t)nb; b += nwarps) {
        const int32_t i = a.big_list[b];
        const SdParticle r = a.rec[i];
        if (r.coef == 0.0f || r.gx1 < r.gx0) continue;  // nothing to deposit
        const int tx0 = r.gx0 / kTile, tx1 = r.gx1 / kTile, ty0 = r.gy0 / kTile, ty1 = r.gy1 / kTile;
        const int nty = ty1 - ty0 + 1, nt = (tx1 - tx0 + 1) * nty;
        for (int u = lane; u < nt; u += 32) {
            const int t = (tx0 + u / nty) * a.ntx + ty0 + u % nty;
            if (scatter)
                a.bpairs[a.btile[t] + atomicAdd(&a.bfill[t], 1u)] = i;
            else
                atomicAdd(&a.btile[t], 1u);
        }
        pairs += (unsigned long long)nt;
    }
    if (!scatter && lane == 0 && pairs)
        atomicAdd(reinterpret_cast<unsigned long long *>(a.big_count + 4), pairs);
}

// Work items per tile of the pairs path: ceil(pairs / kSdBigChunk) (0 for a
// tile no large footprint covers).
__global__ void k_sd_big_items(SdArgs a, int64_t ntiles) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < ntiles) {
        const uint32_t c = a.btile[t + 1] - a.btile[t];
        a.bitem_off[t] = (c + kSdBigChunk - 1) / kSdBigChunk;
    } else if (t == ntiles) {
        a.bitem_off[t] = 0u;
    }
}

// Large footprints, per tile from its own pair list: the work items (a tile's
// pairs in chunks of kSdBigChunk) are taken by a persistent grid; each CTA
// stages 256 records at a time in shared memory (1/h and the normalised
// coefficient computed once per record) and every thread adds their
// contributions to its 4 pixels in registers.  Each warp owns a 16 x 8
// sub-block of the tile (lane l: column l % 8, rows l / 8 + 4 j) and skips
// the records whose footprint box misses it or whose circle misses its nodes
// by more than 1e-4 of h^2 (there every pixel would evaluate q > 1, a weight
// of exactly 0): a footprint of 3 x 3 tiles covers about half of its tiles'
// pixels, so whole sub-blocks drop out.  Per pixel: the offset from the
// footprint's first node in FP32 exactly as the small path forms it
// ((gx - gx0) dx with the integer difference converted exactly), |d| by
// r^2 rsqrt(r^2), and half the spline against twice the coefficient
// (spline_w_half), 0 beyond q = 1.  No per-pixel box test: the footprint box
// holds every node within h of the particle along each axis (the
// truncations of footprint()), so a node outside it lies at q >= 1 and
// weighs exactly 0, up to the FP32 rounding of q near 1 (a weight below
// 1e-18 of the peak; tests/native/sd_cull_check.cu).  A tile of one item adds its values to the pixels
// k_sd_tile wrote; the items of a split tile add theirs with FP64 atomics.
__global__ __launch_bounds__(256) void k_sd_tile_pairs(SdArgs a, int64_t ntiles) {
    __shared__ float4 sa[256];  // rx, ry, 1/h, 2 coef * norm
    __shared__ float4 sb[256];  // gx0, gx1 - gx0, gy0, gy1 - gy0 (exact small integers)
    if (!sd_pairs(a)) return;
    const uint32_t nitems = a.bitem_off[ntiles];
    const int tid = threadIdx.x;
    const float dxf = (float)a.dx;
    const double scale = a.conservative ? 1.0 / (a.dx * a.dx) : 1.0;
    for (uint32_t item = blockIdx.x; item < nitems; item += gridDim.x) {
        int64_t lo = 0, hi = ntiles - 1;  // tile: largest t with bitem_off[t] <= item
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if (a.bitem_off[mid] <= item)
                lo = mid;
            else
                hi = mid - 1;
        }
        const int tile = (int)lo;
        const uint32_t nit = a.bitem_off[tile + 1] - a.bitem_off[tile];
        const uint32_t j = item - a.bitem_off[tile];
        const int tx = tile / a.ntx, ty = tile % a.ntx;
        const int bx0 = tx * kTile + 16 * ((tid >> 5) & 1), by0 = ty * kTile + 8 * (tid >> 6);  // the warp's sub-block
        const int gy = by0 + (tid & 7), gxb = bx0 + ((tid >> 3) & 3);
        const float fgy = (float)gy, fbx0 = (float)bx0, fby0 = (float)by0;
        float fgx[4];
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) fgx[jj] = (float)(gxb + 4 * jj);
        const uint32_t p0 = a.btile[tile] + j * (uint32_t)kSdBigChunk;
        const uint32_t p1 = min(a.btile[tile + 1], p0 + (uint32_t)kSdBigChunk);
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (uint32_t c0 = p0; c0 < p1; c0 += 256) {
            __syncthreads();  // the previous batch is consumed
            if (c0 + tid < p1) {
                const SdParticle r = a.rec[a.bpairs[c0 + tid]];
                sa[tid] = make_float4(r.rx, r.ry, 1.0f / r.h, 2.0f * (r.coef * kKernel2dNorm));
                sb[tid] = make_float4((float)r.gx0, (float)(r.gx1 - r.gx0), (float)r.gy0, (float)(r.gy1 - r.gy0));
            }
            __syncthreads();
            const int m = (int)min(256u, p1 - c0);
            for (int e = 0; e < m; ++e) {
                const float4 pa = sa[e], pb = sb[e];
                if (sd_block_skips(fbx0, fby0, pa, pb, dxf)) continue;  // warp-uniform
                const float oy = fgy - pb.z;  // exact: gy - gy0
                const float ddy = fmaf(-oy, dxf, pa.y);
                const float ddy2 = ddy * ddy;
#pragma unroll
                for (int jj = 0; jj < 4; ++jj) {
                    const float ox = fgx[jj] - pb.x;  // exact: gx - gx0
                    const float ddx = fmaf(-ox, dxf, pa.x);
                    const float r2 = fmaf(ddx, ddx, ddy2);
                    acc[jj] = fmaf(spline_w_half(r2 * rsqrtf(fmaxf(r2, 1e-30f)) * pa.z), pa.w, acc[jj]);
                }
            }
        }
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            const int gx = gxb + 4 * jj;
            if (gx >= a.res || gy >= a.res || acc[jj] == 0.0f) continue;
            double *px = &a.grid[(int64_t)gx * a.res + gy];
            const double v = (double)acc[jj] * scale;
            if (nit == 1)
                *px += v;
            else
                atomicAdd(px, v);
        }
    }
}

// ---- nearest particle of arbitrary points ---------------------------------------
__device__ __forceinline__ double d2_exact_pt(const double *__restrict__ p64, int32_t s, const double t[3],
                                              bool periodic, double box) {
    double acc = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        double d = __dsub_rn(p64[(int64_t)s * 3 + c], t[c]);
        if (periodic && fabs(d) > 0.5 * box) d = -copysign(__dsub_rn(box, fabs(d)), d);
        acc = __dadd_rn(acc, __dmul_rn(d, d));
    }
    return acc;
}

__global__ __launch_bounds__(256) void k_nn_query(const double *__restrict__ targets, int64_t nt, int dim,
                                                  const CellIndex ci, bool periodic, float box_hi, float box_lo,
                                                  const double *__restrict__ framep,
                                                  const int32_t *__restrict__ order,
                                                  const float4 *__restrict__ hi, const float4 *__restrict__ lo,
                                                  const double *__restrict__ pos64, int64_t *__restrict__ nn) {
    const int lane = threadIdx.x & 31;
    const int64_t q = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= nt) return;
    const Frame fr = load_frame(framep);
    const double t[3] = {targets[q * 3], targets[q * 3 + 1], targets[q * 3 + 2]};
    const double c3[3] = {fr.cx, fr.cy, fr.cz};
    float th[3], tl[3];
    for (int d = 0; d < 3; ++d) {
        double r = t[d] - c3[d];
        if (d >= dim) r = 0.0;
        th[d] = (float)r;
        tl[d] = (float)(r - (double)th[d]);
    }
    const float4 h0 = make_float4(th[0], th[1], th[2], 0.f), l0 = make_float4(tl[0], tl[1], tl[2], 0.f);
    const float side = (float)fr.side, half = 0.5f * side;
    // start from the target's level-Lg cell size
    float R = side / (float)(1u << ci.Lg);
    for (int iter = 0; iter < 64; ++iter) {
        int L = (int)floorf(log2f(side / R));
        L = max(0, min(kMaxLevel, L));
        const int M = 1 << L;
        const float scale = (float)M / side;
        const float u[3] = {((h0.x + half) + l0.x) * scale, ((h0.y + half) + l0.y) * scale,
                            ((h0.z + half) + l0.z) * scale};
        const float rc = R * scale * (1.0f + 1e-5f) + 1e-3f + M * 2.4e-7f;
        int cmin[3], cnum[3];
        for (int d = 0; d < 3; ++d) {
            if (d >= dim) {
                cmin[d] = 0;
                cnum[d] = 1;
                continue;
            }
            int lo_c = (int)floorf(u[d] - rc), hi_c = (int)floorf(u[d] + rc);
            if (periodic) {
                if (hi_c - lo_c + 1 >= M) {
                    lo_c = 0;
                    hi_c = M - 1;
                }
            } else {
                lo_c = max(lo_c, 0);
                hi_c = min(hi_c, M - 1);
            }
            cmin[d] = lo_c;
            cnum[d] = max(0, hi_c - lo_c + 1);
        }
        const int ncell = cnum[0] * cnum[1] * cnum[2];
        float best = FLT_MAX;
        int32_t bslot = INT_MAX;
        for (int cb = 0; cb < ncell; cb += 32) {
            const int c = cb + lane;
            uint32_t ca = 0, cbn = 0;
            if (c < ncell) {
                int gx = cmin[0] + c % cnum[0], gy = cmin[1] + (c / cnum[0]) % cnum[1],
                    gz = cmin[2] + c / (cnum[0] * cnum[1]);
                float ddx = fmaxf(0.f, fmaxf((float)gx - u[0], u[0] - (float)(gx + 1)));
                float ddy = fmaxf(0.f, fmaxf((float)gy - u[1], u[1] - (float)(gy + 1)));
                float ddz = fmaxf(0.f, fmaxf((float)gz - u[2], u[2] - (float)(gz + 1)));
                if (dim < 3) ddz = 0.f;
                if (dim < 2) ddy = 0.f;
                if (ddx * ddx + ddy * ddy + ddz * ddz <= rc * rc) {
                    if (periodic) {
                        gx = ((gx % M) + M) % M;
                        gy = ((gy % M) + M) % M;
                        gz = ((gz % M) + M) % M;
                    }
                    if (dim < 3) gz = 0;
                    if (dim < 2) gy = 0;
                    cell_lookup(ci, L, morton3((uint32_t)gx, (uint32_t)gy, (uint32_t)gz), ca, cbn);
                }
            }
            unsigned ne = __ballot_sync(0xffffffffu, cbn > ca);
            while (ne) {
                const int j = __ffs(ne) - 1;
                ne &= ne - 1;
                const uint32_t A = __shfl_sync(0xffffffffu, ca, j), B = __shfl_sync(0xffffffffu, cbn, j);
                for (uint32_t s = A + lane; s < B; s += 32) {
                    const float4 hb = hi[s], lb = lo[s];
                    float3 dd = periodic ? sep_hilo_periodic(h0, l0, hb, lb, box_hi, box_lo) : sep_hilo(h0, l0, hb, lb);
                    const float v = dd.x * dd.x + dd.y * dd.y + dd.z * dd.z;
                    if (v < best || (v == best && (int32_t)s < bslot)) {
                        best = v;
                        bslot = (int32_t)s;
                    }
                }
            }
        }
        const float wbest = warp_min(best);
        if (wbest <= R * R && wbest < FLT_MAX) {
            // exact decision among candidates within 1e-5 of the best (FP64, then index)
            const float lim = wbest * (1.0f + 1e-5f) + 1e-30f;
            double bk = DBL_MAX;
            int32_t bp = INT_MAX;
            for (int cb = 0; cb < ncell; cb += 32) {
                const int c = cb + lane;
                uint32_t ca = 0, cbn = 0;
                if (c < ncell) {
                    int gx = cmin[0] + c % cnum[0], gy = cmin[1] + (c / cnum[0]) % cnum[1],
                        gz = cmin[2] + c / (cnum[0] * cnum[1]);
                    if (periodic) {
                        gx = ((gx % M) + M) % M;
                        gy = ((gy % M) + M) % M;
                        gz = ((gz % M) + M) % M;
                    }
                    if (dim < 3) gz = 0;
                    if (dim < 2) gy = 0;
                    cell_lookup(ci, L, morton3((uint32_t)gx, (uint32_t)gy, (uint32_t)gz), ca, cbn);
                }
                unsigned ne = __ballot_sync(0xffffffffu, cbn > ca);
                while (ne) {
                    const int j = __ffs(ne) - 1;
                    ne &= ne - 1;
                    const uint32_t A = __shfl_sync(0xffffffffu, ca, j), B = __shfl_sync(0xffffffffu, cbn, j);
                    for (uint32_t s = A + lane; s < B; s += 32) {
                        const float4 hb = hi[s], lb = lo[s];
                        float3 dd = periodic ? sep_hilo_periodic(h0, l0, hb, lb, box_hi, box_lo) : sep_hilo(h0, l0, hb, lb);
                        const float v = dd.x * dd.x + dd.y * dd.y + dd.z * dd.z;
                        if (v <= lim) {
                            const double e = d2_exact_pt(pos64, (int32_t)s, t, periodic, fr.side);
                            const int32_t pidx = order[s];
                            if (e < bk || (e == bk && pidx < bp)) {
                                bk = e;
                                bp = pidx;
                            }
                        }
                    }
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double ok = __shfl_xor_sync(0xffffffffu, bk, o);
                const int32_t op = __shfl_xor_sync(0xffffffffu, bp, o);
                if (ok < bk || (ok == bk && op < bp)) {
                    bk = ok;
                    bp = op;
                }
            }
            if (lane == 0) nn[q] = bp;
            return;
        }
        // nothing within R: grow the radius (to the best distance seen if any)
        R = (wbest < FLT_MAX) ? fmaxf(sqrtf(wbest) * 1.001f, R * 1.01f) : R * 2.0f;
    }
    if (lane == 0) nn[q] = -1;
}

}  // namespace mg

using namespace mg;

// (tile, particle) pairs of large footprints the workspace holds: 4 per
// particle (a 2^20 Plummer map of side 8 at 1024^2 has 2.5), at least 2^22,
// at most 2^31 - 1 (the per-tile offsets are 32-bit).
static uint64_t sd_big_capacity(int64_t n) {
    return (uint64_t)std::min<int64_t>(std::max<int64_t>(4 * n, int64_t(1) << 22), (int64_t(1) << 31) - 1);
}

extern "C" size_t mg_surface_density_workspace_bytes(int64_t n, int32_t res) {
    if (n <= 0 || res < 2) return 0;
    const int ntx = (res + kTile - 1) / kTile;
    const int64_t ntiles = (int64_t)ntx * ntx;
    size_t b = 0;
    b += align_up(sizeof(SdParticle) * n);
    b += align_up(sizeof(uint32_t) * (ntiles + 1));
    b += align_up(sizeof(uint32_t) * 4 * n);
    b += align_up(sizeof(int32_t) * n);
    b += align_up(sizeof(uint32_t) * 4);
    b += align_up(sizeof(int32_t) * 4 * n);
    b += align_up(scan_workspace_bytes(ntiles + 1));
    b += align_up(sizeof(uint32_t) * (ntiles + 1));
    b += 3 * align_up(sizeof(uint32_t) * (ntiles + 1));
    b += align_up(sizeof(int32_t) * sd_big_capacity(n));
    return b + 4096;
}

extern "C" int mg_surface_density(const double *pos, const double *h, const double *f, int64_t n, double cx,
                                  double cy, double size, int32_t res, int32_t conservative, double *grid,
                                  void *workspace, size_t workspace_bytes, void *stream_) {
    if (!pos || !h || !f || !grid || n <= 0 || res < 2 || !(size > 0)) return MG_ERR_ARG;
    if (workspace_bytes < mg_surface_density_workspace_bytes(n, res)) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    const int ntx = (res + kTile - 1) / kTile;
    const int64_t ntiles = (int64_t)ntx * ntx;
    Carve w(workspace, workspace_bytes);
    SdArgs a;
    a.pos = pos;
    a.h = h;
    a.f = f;
    a.n = n;
    a.cx = cx;
    a.cy = cy;
    a.size = size;
    a.dx = size / (double)(res - 1);
    a.inv_dx = 1.0 / a.dx;
    a.res = res;
    a.conservative = conservative ? 1 : 0;
    a.ntx = ntx;
    a.rec = w.take<SdParticle>(n);
    a.tile_count = w.take<uint32_t>(ntiles + 1);
    a.ranks = w.take<uint32_t>(4 * n);
    a.big_list = w.take<int32_t>(n);
    a.big_count = w.take<uint32_t>(8);
    a.pairs = w.take<int32_t>(4 * n);
    void *scan_ws = w.take<char>(scan_workspace_bytes(ntiles + 1));
    a.item_off = w.take<uint32_t>(ntiles + 1);
    a.grid = grid;
    a.btile = w.take<uint32_t>(ntiles + 1);
    a.bfill = w.take<uint32_t>(ntiles + 1);
    a.bitem_off = w.take<uint32_t>(ntiles + 1);
    a.bcap = sd_big_capacity(n);
    a.bpairs = w.take<int32_t>(a.bcap);
    if (!w.ok()) return MG_ERR_ARG;
    MG_CUDA(cudaMemsetAsync(a.tile_count, 0, sizeof(uint32_t) * (ntiles + 1), st));
    MG_CUDA(cudaMemsetAsync(a.big_count, 0, sizeof(uint32_t) * 8, st));
    MG_CUDA(cudaMemsetAsync(a.btile, 0, sizeof(uint32_t) * (ntiles + 1), st));
    MG_CUDA(cudaMemsetAsync(a.bfill, 0, sizeof(uint32_t) * (ntiles + 1), st));
    const unsigned nb = (unsigned)((n + 255) / 256);
    k_sd_prep<<<nb, 256, 0, st>>>(a);
    MG_CHECK_LAUNCH();
    int dev = 0, nsm = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (conservative) {
        k_sd_cons_norm<<<(unsigned)(nsm * 8), 256, 0, st>>>(a);
        MG_CHECK_LAUNCH();
    }
    int rc = exclusive_scan_u32(a.tile_count, a.tile_count, ntiles + 1, scan_ws, st);
    if (rc) return rc;
    k_sd_scatter<<<nb, 256, 0, st>>>(a);
    MG_CHECK_LAUNCH();
    // crowded tiles are split into chunks (their CTAs add atomically into the
    // zeroed grid); one CTA per work item, grid sized for the most items possible
    MG_CUDA(cudaMemsetAsync(grid, 0, sizeof(double) * (size_t)res * (size_t)res, st));
    k_sd_items<<<(unsigned)((ntiles + 1 + 255) / 256), 256, 0, st>>>(a, ntiles);
    MG_CHECK_LAUNCH();
    rc = exclusive_scan_u32(a.item_off, a.item_off, ntiles + 1, scan_ws, st);
    if (rc) return rc;
    const int64_t max_items = ntiles + (4 * n) / kSdChunk + 1;
    k_sd_tile<<<(unsigned)max_items, 256, 0, st>>>(a, ntiles);
    MG_CHECK_LAUNCH();
    // large footprints: per-tile pairs when they fit the buffer (decided on
    // the device from the count), else the gather or the FP64-atomic path
    k_sd_big_pairs<<<(unsigned)(nsm * 8), 256, 0, st>>>(a, 0);
    MG_CHECK_LAUNCH();
    rc = exclusive_scan_u32(a.btile, a.btile, ntiles + 1, scan_ws, st);
    if (rc) return rc;
    k_sd_big_pairs<<<(unsigned)(nsm * 8), 256, 0, st>>>(a, 1);
    MG_CHECK_LAUNCH();
    k_sd_big_items<<<(unsigned)((ntiles + 1 + 255) / 256), 256, 0, st>>>(a, ntiles);
    MG_CHECK_LAUNCH();
    rc = exclusive_scan_u32(a.bitem_off, a.bitem_off, ntiles + 1, scan_ws, st);
    if (rc) return rc;
    k_sd_tile_pairs<<<(unsigned)(nsm * 8), 256, 0, st>>>(a, ntiles);
    MG_CHECK_LAUNCH();
    k_sd_tile_big<<<(unsigned)ntiles, 256, 0, st>>>(a);
    MG_CHECK_LAUNCH();
    k_sd_big<<<(unsigned)(nsm * 4), 256, 0, st>>>(a);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" size_t mg_nn_query_workspace_bytes(int64_t nt) { return nt > 0 ? 256 : 0; }

extern "C" int mg_nn_query(const mg_cells *c, const double *targets, int64_t nt, int64_t *nn, void *workspace,
                           size_t workspace_bytes, void *stream_) {
    (void)workspace;
    (void)workspace_bytes;
    if (!c || !targets || !nn || nt <= 0) return MG_ERR_ARG;
    const float box_hi = (float)c->boxsize;
    const float box_lo = (float)(c->boxsize - (double)box_hi);
    CellIndex ci;
    ci.Lg = c->grid_level;
    ci.keys = c->keys;
    ci.cs = c->cell_start;
    const bool use_bricks = c->brick_of && c->bricks && c->brick_capacity > 0;
    ci.brick_of = use_bricks ? c->brick_of : nullptr;
    ci.bricks = use_bricks ? c->bricks : nullptr;
    k_nn_query<<<(unsigned)((nt + 7) / 8), 256, 0, as_stream(stream_)>>>(
        targets, nt, c->dim, ci, c->boxsize > 0, box_hi, box_lo, c->frame, c->order, reinterpret_cast<const float4 *>(c->pos_hi), reinterpret_cast<const float4 *>(c->pos_lo),
        c->pos64, nn);
    MG_CHECK_LAUNCH();
    return MG_OK;
}
