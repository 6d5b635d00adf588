// Spatial index: bounding frame, 63-bit Morton keys, LSD radix sort of
// (key, particle) pairs, slot-order FP32 hi/lo positions and the dense cell
// table.  This replaces cKDTree construction (src/meshoid/Meshoid.py:142-145);
// the neighbour query itself lives in mg_knn.cu.
#include <cstdio>

#include "mg_common.cuh"
#include "mg_scan.cuh"

namespace mg {

constexpr int kRsThreads = 256;
constexpr int kRsRounds = 8;
constexpr int kRsTile = kRsThreads * kRsRounds;  // 2048 pairs per block
constexpr int kRsPasses = (64 - kSortLowBit + 7) / 8;  // 7 passes of 8 bits

// ---- bounding frame ---------------------------------------------------------

__global__ void k_bbox_partial(const double *__restrict__ pos, int64_t n, int dim,
                               double *__restrict__ partial) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        for (int a = 0; a < dim; ++a) {
            double v = pos[i * dim + a];
            lo[a] = fmin(lo[a], v);
            hi[a] = fmax(hi[a], v);
        }
    }
    __shared__ double s[6][256];
    for (int a = 0; a < 3; ++a) {
        s[a][threadIdx.x] = lo[a];
        s[3 + a][threadIdx.x] = hi[a];
    }
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            for (int a = 0; a < 3; ++a) {
                s[a][threadIdx.x] = fmin(s[a][threadIdx.x], s[a][threadIdx.x + o]);
                s[3 + a][threadIdx.x] = fmax(s[3 + a][threadIdx.x], s[3 + a][threadIdx.x + o]);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 6) partial[blockIdx.x * 6 + threadIdx.x] = s[threadIdx.x][0];
}

__global__ __launch_bounds__(256) void k_frame(const double *__restrict__ partial, int nparts, int dim,
                                               double boxsize, double *__restrict__ frame) {
    __shared__ double s[6][256];
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int b = threadIdx.x; b < nparts; b += blockDim.x)
        for (int a = 0; a < 3; ++a) {
            lo[a] = fmin(lo[a], partial[b * 6 + a]);
            hi[a] = fmax(hi[a], partial[b * 6 + 3 + a]);
        }
    for (int a = 0; a < 3; ++a) {
        s[a][threadIdx.x] = lo[a];
        s[3 + a][threadIdx.x] = hi[a];
    }
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int a = 0; a < 3; ++a) {
                s[a][threadIdx.x] = fmin(s[a][threadIdx.x], s[a][threadIdx.x + o]);
                s[3 + a][threadIdx.x] = fmax(s[3 + a][threadIdx.x], s[3 + a][threadIdx.x + o]);
            }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    for (int a = 0; a < 3; ++a) {
        lo[a] = a < dim ? s[a][0] : 0.0;
        hi[a] = a < dim ? s[3 + a][0] : 0.0;
    }
    double side;
    if (boxsize > 0) {
        lo[0] = lo[1] = lo[2] = 0.0;
        side = boxsize;
    } else {
        side = 0.0;
        for (int a = 0; a < dim; ++a) side = fmax(side, hi[a] - lo[a]);
        double mag = 0.0;
        for (int a = 0; a < dim; ++a) mag = fmax(mag, fmax(fabs(lo[a]), fabs(hi[a])));
        // pad so the maximum coordinate maps strictly inside the cube
        side = side * (1.0 + 1.0 / 1048576.0) + mag * 1e-12 + 1e-300;
        if (!(side > 0.0)) side = 1.0;
    }
    frame[0] = lo[0];
    frame[1] = lo[1];
    frame[2] = lo[2];
    frame[3] = side;
    frame[4] = 1.0 / side;
    for (int a = 0; a < 3; ++a) frame[5 + a] = (a < dim) ? lo[a] + 0.5 * side : 0.0;
}

// ---- keys ------------------------------------------------------------------

__global__ void k_keys(const double *__restrict__ pos, int64_t n, int dim,
                       const double *__restrict__ framep, uint64_t *__restrict__ keys,
                       int32_t *__restrict__ vals) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    Frame f = load_frame(framep);
    const double o[3] = {f.ox, f.oy, f.oz};
    const double scale = f.inv_side * (double)(1u << kKeyBits);
    uint32_t c[3] = {0, 0, 0};
    for (int a = 0; a < dim; ++a) {
        double t = (pos[i * dim + a] - o[a]) * scale;
        t = fmin(fmax(t, 0.0), (double)((1u << kKeyBits) - 1));
        c[a] = (uint32_t)t;
    }
    keys[i] = morton3(c[0], c[1], c[2]);
    vals[i] = (int32_t)i;
}

// ---- LSD radix sort (stable), 8-bit digits ------------------------------------

__global__ __launch_bounds__(kRsThreads) void k_radix_hist(const uint64_t *__restrict__ kin,
                                                           int64_t n, int shift,
                                                           uint32_t *__restrict__ counts, int nb) {
    __shared__ uint32_t h[256];
    const int tid = threadIdx.x, lane = tid & 31;
    h[tid] = 0;
    __syncthreads();
    const int64_t t0 = (int64_t)blockIdx.x * kRsTile;
    for (int r = 0; r < kRsRounds; ++r) {
        int64_t i = t0 + r * kRsThreads + tid;
        uint32_t d = i < n ? (uint32_t)((kin[i] >> shift) & 255u) : 256u;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        if (d < 256u && lane == __ffs(peers) - 1) atomicAdd(&h[d], (uint32_t)__popc(peers));
    }
    __syncthreads();
    counts[(int64_t)tid * nb + blockIdx.x] = h[tid];
}

__global__ __launch_bounds__(kRsThreads) void k_radix_scatter(
    const uint64_t *__restrict__ kin, const int32_t *__restrict__ vin, uint64_t *__restrict__ kout,
    int32_t *__restrict__ vout, int64_t n, int shift, const uint32_t *__restrict__ offsets, int nb) {
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[kRsThreads / 32][256];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    base[tid] = offsets[(int64_t)tid * nb + blockIdx.x];
    const int64_t t0 = (int64_t)blockIdx.x * kRsTile;
    for (int r = 0; r < kRsRounds; ++r) {
#pragma unroll
        for (int w = 0; w < kRsThreads / 32; ++w) wcnt[w][tid] = 0;
        __syncthreads();
        const int64_t i = t0 + r * kRsThreads + tid;
        const bool valid = i < n;
        uint64_t key = valid ? kin[i] : 0ull;
        int32_t val = valid ? vin[i] : 0;
        uint32_t d = valid ? (uint32_t)((key >> shift) & 255u) : 256u;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] = (uint32_t)__popc(peers);
        __syncthreads();
        uint32_t run = base[tid];
#pragma unroll
        for (int w = 0; w < kRsThreads / 32; ++w) {
            uint32_t c = wcnt[w][tid];
            wcnt[w][tid] = run;
            run += c;
        }
        base[tid] = run;
        __syncthreads();
        if (valid) {
            uint32_t p = wcnt[warp][d] + (uint32_t)rank;
            kout[p] = key;
            vout[p] = val;
        }
        __syncthreads();
    }
}

// ---- slot-order positions -----------------------------------------------------

__global__ void k_slot_positions(const double *__restrict__ pos, int64_t n, int dim,
                                 const double *__restrict__ framep,
                                 const int32_t *__restrict__ order, int32_t *__restrict__ rank,
                                 float4 *__restrict__ hi, float4 *__restrict__ lo,
                                 double *__restrict__ pos64) {
    int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    Frame f = load_frame(framep);
    const int32_t p = order[s];
    rank[p] = (int32_t)s;
    double x[3] = {0.0, 0.0, 0.0};
    for (int a = 0; a < dim; ++a) x[a] = pos[(int64_t)p * dim + a];
    const double c[3] = {f.cx, f.cy, f.cz};
    float h[3], l[3];
    for (int a = 0; a < 3; ++a) {
        double r = x[a] - c[a];
        h[a] = (float)r;
        l[a] = (float)(r - (double)h[a]);
        pos64[s * 3 + a] = x[a];
    }
    hi[s] = make_float4(h[0], h[1], h[2], 0.0f);
    lo[s] = make_float4(l[0], l[1], l[2], 0.0f);
}

// ---- dense cell table ---------------------------------------------------------

__global__ void k_cell_count(const uint64_t *__restrict__ keys, int64_t n, int shift,
                             uint32_t *__restrict__ count) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    uint64_t c = i < n ? (keys[i] >> shift) : ~0ull;
    unsigned peers = __match_any_sync(0xffffffffu, c);
    if (i < n && lane == __ffs(peers) - 1) atomicAdd(&count[c], (uint32_t)__popc(peers));
}

// ---- bricks: refinement tables below the dense level ----------------------------
// Level m bricks cover cells at level Lg + 3m holding more than T particles;
// each stores the first slots of its 512 descendants at level Lg + 3m + 3, the
// child brick of each descendant (-1: none) and its own slot range.  Built
// level by level without host synchronisation: lvl[2m], lvl[2m+1] hold the
// first brick id and the brick count of level m on the device.

inline int brick_levels(int Lg) {
    int m = 0;
    for (int l = Lg; l + 3 <= kMaxLevel; l += 3) ++m;
    return m;
}

__global__ void k_brick_top_count(const uint32_t *__restrict__ cs, int64_t ncell, int T,
                                  uint32_t *__restrict__ flags) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c < ncell) flags[c] = (cs[c + 1] - cs[c] > (uint32_t)T) ? 1u : 0u;
    if (c == ncell) flags[c] = 0u;
}

__global__ void k_brick_top_assign(const uint32_t *__restrict__ cs, const uint32_t *__restrict__ scanned,
                                   int64_t ncell, int cap, int32_t *__restrict__ brick_of,
                                   uint32_t *__restrict__ bricks, int32_t *__restrict__ lvl) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c < ncell) {
        const uint32_t id = scanned[c];
        const bool big = scanned[c + 1] != id;
        if (big && id < (uint32_t)cap) {
            brick_of[c] = (int32_t)id;
            uint32_t *br = bricks + (size_t)id * kBrickWords;
            br[kBrickRange] = cs[c];
            br[kBrickRange + 1] = cs[c + 1];
        } else {
            brick_of[c] = -1;
        }
    }
    if (c == 0) {
        lvl[0] = 0;
        lvl[1] = (int32_t)min(scanned[ncell], (uint32_t)cap);
    }
}

// start[s] = range end, child[s] = -1 for every brick of level m
__global__ void k_brick_init(uint32_t *__restrict__ bricks, const int32_t *__restrict__ lvl, int m) {
    const int base = lvl[2 * m], nb = lvl[2 * m + 1];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)nb * 513;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int b = base + (int)(i / 513), s = (int)(i % 513);
        uint32_t *br = bricks + (size_t)b * kBrickWords;
        br[s] = br[kBrickRange + 1];
        if (s < 512) br[kBrickChild + s] = 0xffffffffu;
    }
}

// particle p opens a descendant of its level-m brick: record the first slot
__global__ void k_brick_mark(const uint64_t *__restrict__ keys, int64_t n, int Lg, const int32_t *__restrict__ brick_of,
                             uint32_t *__restrict__ bricks, int m) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint64_t key = keys[p];
    int br = brick_of[key >> (3 * (kKeyBits - Lg))];
    for (int l = 0; l < m && br >= 0; ++l) {
        const uint32_t sub = (uint32_t)((key >> (3 * (kKeyBits - (Lg + 3 * (l + 1))))) & 511ull);
        br = (int)bricks[(size_t)br * kBrickWords + kBrickChild + sub];
    }
    if (br < 0) return;
    uint32_t *b = bricks + (size_t)br * kBrickWords;
    const int shift = 3 * (kKeyBits - (Lg + 3 * (m + 1)));
    const uint32_t sub = (uint32_t)((key >> shift) & 511ull);
    const bool first = (uint32_t)p == b[kBrickRange] || ((keys[p - 1] >> shift) & 511ull) != sub;
    if (first) b[sub] = (uint32_t)p;
}

// empty descendants start where the next non-empty one does; count big ones
__global__ void k_brick_fill(uint32_t *__restrict__ bricks, const int32_t *__restrict__ lvl, int m, int T,
                             uint32_t *__restrict__ nchild) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= lvl[2 * m + 1]) return;
    uint32_t *b = bricks + (size_t)(lvl[2 * m] + i) * kBrickWords;
    uint32_t nxt = b[512], cnt = 0;
    for (int s = 511; s >= 0; --s) {
        const uint32_t v = min(b[s], nxt);
        b[s] = v;
        cnt += (nxt - v > (uint32_t)T) ? 1u : 0u;
        nxt = v;
    }
    nchild[i] = cnt;
}

__global__ void k_brick_children(uint32_t *__restrict__ bricks, int32_t *__restrict__ lvl, int m, int T, int cap,
                                 const uint32_t *__restrict__ scanned) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int base = lvl[2 * m], nb = lvl[2 * m + 1];
    const int nbase = base + nb;
    if (i == 0) {
        lvl[2 * (m + 1)] = nbase;
        lvl[2 * (m + 1) + 1] = (int32_t)min((uint32_t)max(cap - nbase, 0), scanned[nb]);
    }
    if (i >= nb) return;
    uint32_t *b = bricks + (size_t)(base + i) * kBrickWords;
    int id = nbase + (int)scanned[i];
    for (int s = 0; s < 512; ++s) {
        if (b[s + 1] - b[s] > (uint32_t)T) {
            if (id < cap) {
                b[kBrickChild + s] = (uint32_t)id;
                uint32_t *c = bricks + (size_t)id * kBrickWords;
                c[kBrickRange] = b[s];
                c[kBrickRange + 1] = b[s + 1];
            }
            ++id;
        }
    }
}

}  // namespace mg

using namespace mg;

// ---- generic stable sort of (u64 key, i32 value) pairs by bits [bit0, bit0 + nbits)
namespace mg {

size_t radix_sort_workspace_bytes(int64_t n) {
    const int64_t nb = (n + kRsTile - 1) / kRsTile;
    return align_up(sizeof(uint64_t) * (size_t)n) + align_up(sizeof(int32_t) * (size_t)n) +
           align_up(sizeof(uint32_t) * 256 * (size_t)nb) + align_up(scan_workspace_bytes(256 * nb)) + 1024;
}

int radix_sort_pairs(uint64_t *keys, int32_t *vals, int64_t n, int bit0, int nbits, void *ws, size_t wsb,
                     cudaStream_t st) {
    if (n <= 1 || nbits <= 0) return MG_OK;
    if (n > 0x7fffffffll || wsb < radix_sort_workspace_bytes(n)) return MG_ERR_ARG;
    const int64_t nb = (n + kRsTile - 1) / kRsTile;
    Carve w(ws, wsb);
    uint64_t *kping = w.take<uint64_t>((size_t)n);
    int32_t *vping = w.take<int32_t>((size_t)n);
    uint32_t *counts = w.take<uint32_t>(256 * (size_t)nb);
    void *scan_ws = w.take<char>(scan_workspace_bytes(256 * nb));
    if (!w.ok()) return MG_ERR_ARG;
    uint64_t *kin = keys, *kout = kping;
    int32_t *vin = vals, *vout = vping;
    const int passes = (nbits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        const int shift = bit0 + 8 * p;
        k_radix_hist<<<(unsigned)nb, kRsThreads, 0, st>>>(kin, n, shift, counts, (int)nb);
        MG_CHECK_LAUNCH();
        int rc = exclusive_scan_u32(counts, counts, 256 * nb, scan_ws, st);
        if (rc) return rc;
        k_radix_scatter<<<(unsigned)nb, kRsThreads, 0, st>>>(kin, vin, kout, vout, n, shift, counts, (int)nb);
        MG_CHECK_LAUNCH();
        uint64_t *tk = kin; kin = kout; kout = tk;
        int32_t *tv = vin; vin = vout; vout = tv;
    }
    if (kin != keys) {
        MG_CUDA(cudaMemcpyAsync(keys, kin, sizeof(uint64_t) * (size_t)n, cudaMemcpyDeviceToDevice, st));
        MG_CUDA(cudaMemcpyAsync(vals, vin, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    }
    return MG_OK;
}

}  // namespace mg

extern "C" int32_t mg_brick_capacity(int64_t n, int grid_level, int threshold) {
    if (n <= 0 || threshold < 1 || grid_level < 1) return 0;
    const int64_t lv = brick_levels(grid_level);
    int64_t cap = lv * (n / threshold) + 16;
    if (cap > (1 << 30)) cap = 1 << 30;
    return (int32_t)cap;
}

// Finest level with 8^(L+1) <= 4n (about 2-16 particles per dense cell), at
// most 9: measured best or within 2% of the best with level_bias 1 for
// Plummer, clump-mixture and uniform sets of 2^18..2^24 particles.
extern "C" int mg_default_grid_level(int64_t n) {
    int L = 1;
    while (L < 9 && (int64_t)1 << (3 * (L + 1)) <= 4 * n) ++L;
    return L;
}

static size_t cell_table_entries(int L) { return ((size_t)1 << (3 * L)) + 1; }

extern "C" size_t mg_build_cells_workspace_bytes(int64_t n, int grid_level) {
    if (n <= 0 || grid_level < 1 || grid_level > 9) return 0;
    const int64_t nb = (n + kRsTile - 1) / kRsTile;
    size_t b = 0;
    b += align_up(sizeof(uint64_t) * n);           // keys ping buffer
    b += align_up(sizeof(int32_t) * n);            // vals ping buffer
    b += align_up(sizeof(uint32_t) * 256 * nb);    // digit counts / offsets
    b += align_up(scan_workspace_bytes(256 * nb));
    b += align_up(scan_workspace_bytes(cell_table_entries(grid_level)));
    b += align_up(sizeof(double) * 6 * 1024);      // bbox partials
    // bricks: flags over the dense cells, per-brick child counts, level table
    b += align_up(sizeof(uint32_t) * (cell_table_entries(grid_level) + 1));
    const int64_t cap = mg_brick_capacity(n, grid_level, 64);  // smallest threshold we size for
    b += align_up(sizeof(uint32_t) * (cap + 1));
    b += align_up(scan_workspace_bytes(cap + 1));
    b += align_up(sizeof(int32_t) * 64);
    return b + 4096;
}

extern "C" int mg_build_cells(const double *pos, mg_cells *c, void *workspace,
                              size_t workspace_bytes, void *stream_) {
    if (!pos || !c || c->n <= 0 || c->dim < 1 || c->dim > 3 || c->grid_level < 1 ||
        c->grid_level > 9 || !c->frame || !c->keys || !c->order || !c->rank || !c->pos_hi ||
        !c->pos_lo || !c->pos64 || !c->cell_start)
        return MG_ERR_ARG;
    if (c->n >= ((int64_t)1 << 31) - 1) return MG_ERR_UNSUPPORTED;
    const int64_t n = c->n;
    const int dim = c->dim;
    cudaStream_t st = as_stream(stream_);
    if (workspace_bytes < mg_build_cells_workspace_bytes(n, c->grid_level)) return MG_ERR_ARG;
    Carve w(workspace, workspace_bytes);
    const int64_t nb = (n + kRsTile - 1) / kRsTile;
    uint64_t *kping = w.take<uint64_t>(n);
    int32_t *vping = w.take<int32_t>(n);
    uint32_t *counts = w.take<uint32_t>(256 * nb);
    void *scan_ws = w.take<char>(scan_workspace_bytes(256 * nb));
    void *scan_ws2 = w.take<char>(scan_workspace_bytes(cell_table_entries(c->grid_level)));
    double *partial = w.take<double>(6 * 1024);
    if (!w.ok()) return MG_ERR_ARG;

    int nparts = (int)((n + 255) / 256);
    if (nparts > 1024) nparts = 1024;
    k_bbox_partial<<<nparts, 256, 0, st>>>(pos, n, dim, partial);
    MG_CHECK_LAUNCH();
    k_frame<<<1, 256, 0, st>>>(partial, nparts, dim, c->boxsize, c->frame);
    MG_CHECK_LAUNCH();
    const int tb = 256;
    const int64_t gb = (n + tb - 1) / tb;
    // Keys land in the ping buffer; after an odd number of passes the sorted
    // result is in the caller's arrays.
    static_assert(kRsPasses % 2 == 1, "pass count parity decides the output buffer");
    k_keys<<<gb, tb, 0, st>>>(pos, n, dim, c->frame, kping, vping);
    MG_CHECK_LAUNCH();
    uint64_t *kin = kping, *kout = c->keys;
    int32_t *vin = vping, *vout = c->order;
    for (int p = 0; p < kRsPasses; ++p) {
        const int shift = kSortLowBit + 8 * p;
        k_radix_hist<<<nb, kRsThreads, 0, st>>>(kin, n, shift, counts, (int)nb);
        MG_CHECK_LAUNCH();
        int rc = exclusive_scan_u32(counts, counts, 256 * nb, scan_ws, st);
        if (rc) return rc;
        k_radix_scatter<<<nb, kRsThreads, 0, st>>>(kin, vin, kout, vout, n, shift, counts, (int)nb);
        MG_CHECK_LAUNCH();
        uint64_t *tk = kin; kin = kout; kout = tk;
        int32_t *tv = vin; vin = vout; vout = tv;
    }
    k_slot_positions<<<gb, tb, 0, st>>>(pos, n, dim, c->frame, c->order, c->rank,
                                        reinterpret_cast<float4 *>(c->pos_hi),
                                        reinterpret_cast<float4 *>(c->pos_lo), c->pos64);
    MG_CHECK_LAUNCH();
    const size_t ncell = cell_table_entries(c->grid_level);
    MG_CUDA(cudaMemsetAsync(c->cell_start, 0, sizeof(uint32_t) * ncell, st));
    k_cell_count<<<gb, tb, 0, st>>>(c->keys, n, 3 * (kKeyBits - c->grid_level), c->cell_start);
    MG_CHECK_LAUNCH();
    int rc = exclusive_scan_u32(c->cell_start, c->cell_start, (int64_t)ncell, scan_ws2, st);
    if (rc) return rc;
    if (!c->brick_of || !c->bricks || c->brick_capacity <= 0) return MG_OK;
    // ---- bricks ----
    const int T = c->brick_threshold > 0 ? c->brick_threshold : 256;
    const int cap = c->brick_capacity;
    // the workspace holds per-brick counters for the capacity at threshold 64
    if (cap > mg_brick_capacity(n, c->grid_level, 64)) return MG_ERR_ARG;
    const int64_t ndense = (int64_t)ncell - 1;
    uint32_t *flags = w.take<uint32_t>(ncell + 1);
    uint32_t *nchild = w.take<uint32_t>((size_t)cap + 1);
    void *scan_ws3 = w.take<char>(scan_workspace_bytes((int64_t)cap + 1));
    int32_t *lvl = w.take<int32_t>(64);
    if (!w.ok()) return MG_ERR_ARG;
    k_brick_top_count<<<(unsigned)((ndense + 1 + 255) / 256), 256, 0, st>>>(c->cell_start, ndense, T, flags);
    MG_CHECK_LAUNCH();
    rc = exclusive_scan_u32(flags, flags, ndense + 1, scan_ws2, st);
    if (rc) return rc;
    k_brick_top_assign<<<(unsigned)((ndense + 255) / 256), 256, 0, st>>>(c->cell_start, flags, ndense, cap,
                                                                          c->brick_of, c->bricks, lvl);
    MG_CHECK_LAUNCH();
    int dev = 0, nsm = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int levels = brick_levels(c->grid_level);
    const unsigned bb = (unsigned)((cap + 127) / 128);
    for (int m = 0; m < levels; ++m) {
        k_brick_init<<<nsm * 8, 256, 0, st>>>(c->bricks, lvl, m);
        MG_CHECK_LAUNCH();
        k_brick_mark<<<gb, tb, 0, st>>>(c->keys, n, c->grid_level, c->brick_of, c->bricks, m);
        MG_CHECK_LAUNCH();
        k_brick_fill<<<bb, 128, 0, st>>>(c->bricks, lvl, m, T, nchild);
        MG_CHECK_LAUNCH();
        if (m + 1 < levels) {
            rc = exclusive_scan_u32(nchild, nchild, (int64_t)cap + 1, scan_ws3, st);
            if (rc) return rc;
            k_brick_children<<<bb, 128, 0, st>>>(c->bricks, lvl, m, T, cap, nchild);
            MG_CHECK_LAUNCH();
        }
    }
    return MG_OK;
}

extern "C" const char *mg_status_string(int s) {
    switch (s) {
        case MG_OK: return "ok";
        case MG_ERR_ARG: return "invalid argument";
        case MG_ERR_CUDA: return "CUDA error";
        case MG_ERR_NOT_CONVERGED: return "search pass cap reached for some queries";
        case MG_ERR_UNSUPPORTED: return "unsupported size or parameter";
        case MG_ERR_NOALLOC_LIMIT:
            return "more queries than the fixed scratch of the no-allocation entry point holds "
                   "(MG_NOALLOC_MAX_QUERIES); use mg_grad_sweep with a workspace";
        default: return "unknown status";
    }
}

extern "C" int mg_version(void) { return 100; }

#include <atomic>
static std::atomic<long long> g_launches{0};
void mg::count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
extern "C" int64_t mg_launch_count(void) { return (int64_t)g_launches.load(std::memory_order_relaxed); }
