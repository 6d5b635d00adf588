// Neighbour search + smoothing-length solve, the plain seed, and the per-row
// FP64 distance accessor.
//
// Replaces cKDTree.query(pos[mask], des_ngb) (src/meshoid/Meshoid.py:157)
// followed by HsmlIter (src/meshoid/kernel_density.py:15-56).
//
// Search, first pass (k_knn_group): one thread per query over the particles
// staged once per block of 128 consecutive queries; it accepts a query only
// when an error bound proves its set exact, and queues the rest.
//
// Search, warp passes (k_knn_hsml; every pass for periodic boxes or k > 32):
// the query's radius R comes from a seed or the queue.  The level L with cell
// side s_L >= R (or R / 2) is chosen, the level-L cells that meet the sphere
// of radius R are looked up (dense table for L <= grid_level, refinement
// tables or a binary search of the Morton keys below), and every particle of
// those cells with FP32 d^2 <= R^2 is appended to a per-warp shared-memory
// buffer.  Fewer than k hits, or more than the buffer holds, re-queues the
// query with a corrected radius (work queue over passes).  The k smallest are
// picked by a 32-bucket histogram in (d/R)^dim; entries within 1e-5
// (relative, in d^2) of the k-th distance are re-decided with exact FP64
// distances and the particle index, so the set equals the k smallest by
// (FP64 d^2, index).  A query whose cells hold more than 2048 particles (a
// sparse query next to a dense clump) is handed with its cell list to a
// block-wide kernel, so that no warp scans a long list alone while the grid
// waits for it.
//
// h: norm * sum_j W(d_j/h) = k (norm = 32/3, 40/7, 8/3 in 3/2/1-D), solved by
// bracketed Newton (bisection fallback), one thread per query, on the k FP32
// distances of its row.  The function is C^2 and increasing in h, so the root
// is unique; the reference bisects to |n - k| <= 1e-13 and outputs the
// midpoint, i.e. the same root.
#include <algorithm>
#include <atomic>
#include <cfloat>

#include <cooperative_groups.h>

#include "mg_common.cuh"
#include "mg_grad2.cuh"
#include "mg_hsml.cuh"
#include "mg_refine.cuh"

namespace mg {

namespace cg = cooperative_groups;

constexpr int kKnnWarps = 8;     // warps per block
constexpr float kBandEps = 1e-5f;
// The search loop's dynamic-trip-count loops are kept rolled: the kernel is
// bound by instruction issue and fetch (32 warps per SM at different points of
// a long loop body), and unrolled copies of these loops made it 14% slower
// (2^22 Plummer, first pass).
#define KNN_LOOP_HINT _Pragma("unroll 1")
#ifdef MG_KNN_SELECT_NOINLINE
#define KNN_SELECT_INLINE __noinline__
#else
#define KNN_SELECT_INLINE __forceinline__
#endif
#ifndef MG_KNN_MINBLOCKS
#define MG_KNN_MINBLOCKS 4
#endif
constexpr int kKnnMinBlocks = MG_KNN_MINBLOCKS;  // resident blocks per SM the register budget is cut for
#ifndef MG_KNN_CHUNK
#define MG_KNN_CHUNK 32
#endif
#ifndef MG_KNN_SPLIT
#define MG_KNN_SPLIT 192
#endif
constexpr int kChunk = MG_KNN_CHUNK;  // consecutive queries per warp on the first pass
constexpr int kSplit = MG_KNN_SPLIT;  // cells holding more particles than this are split when they straddle the sphere
constexpr int kList = 128;       // scan-list capacity per warp
constexpr int kScanLimit = 1 << 20;  // scan-list particles above which a first radius is halved unscanned
// Queries per run dealt to a warp of the warp passes in turn (0: one
// contiguous run per warp).  The queue's cost is uneven (the slowest warp of
// a contiguous split took 1.8x the mean), and balance pays more than the
// cell-box reuse of long runs: search + h at 2^22 (Plummer / clump mixture)
// 10.83 / 19.82 ms with contiguous runs, 10.70 / 19.23 with runs of 4,
// 10.68 / 18.38 with single queries.
#ifndef MG_KNN_WCHUNK
#define MG_KNN_WCHUNK 1
#endif
#ifndef MG_KNN_HEAVY
#define MG_KNN_HEAVY 2048
#endif
constexpr int kHeavy = MG_KNN_HEAVY;  // scan-list particles above which a query goes to the block-wide path
constexpr int kHeavyItem = 2 * kList + 4;  // int32 words per queued heavy query: qi, nlist, pa[], off[]
constexpr int kHeavyThreads = 256;
constexpr int kHeavyBins = 1024;
constexpr int kHeavyCap = 1 << 16;   // heavy queries queued per pass (beyond: scanned by their warp)

struct KnnArgs {
    CellIndex ci;
    int64_t n;
    int dim, Lg;
    bool periodic;
    float box_hi, box_lo;
    double box64;  // the box side (periodic), FP64
    const double *frame;
    const uint64_t *keys;
    const uint32_t *cell_start;
    const int32_t *order;
    const float4 *hi;
    const float4 *lo;
    const double *pos64;
    const int32_t *queries;
    int64_t nq;
    int k;
    const float *seed_h;
    float radius_factor;
    float *radius;
    float *rlo;  // largest radius seen with fewer than k particles (0: none)
    float *rhi;  // smallest radius seen with too many particles to scan (0: none)
    int32_t *ngb;
    float *hsml;
    int32_t *qstatus;
    const int32_t *qin;          // nullptr on the first pass
    const int32_t *qin_count;
    int32_t *qout;
    int32_t *qout_count;
    int64_t *stats;
    int last_pass;
    int level_bias;  // search cells of side s with s >= R / 2^level_bias
    int32_t *heavy;        // heavy-query items of this pass (kHeavyItem words each)
    int32_t *heavy_count;  // items queued this pass (may exceed heavy_cap: the excess was not queued)
    int32_t *heavy_next;   // next item to take (block-wide path)
    int heavy_cap;
};

// Slot range [a, b) of the level-L cell with coordinates (cx, cy, cz).
#ifdef MG_KNN_LOOKUP_NOINLINE
#define KNN_LOOKUP_INLINE __noinline__
#else
#define KNN_LOOKUP_INLINE __forceinline__
#endif
__device__ KNN_LOOKUP_INLINE void cell_range(const CellIndex &ci, int L, uint32_t cx, uint32_t cy, uint32_t cz,
                                             uint32_t &a, uint32_t &b) {
    cell_lookup(ci, L, morton3(cx, cy, cz), a, b);
}

__device__ __forceinline__ float bucket_of(float t, int dim) {
    // t = d^2 / R^2 in [0, 1]; buckets uniform in enclosed volume (d/R)^dim
    float v = dim == 3 ? t * sqrtf(t) : (dim == 2 ? t : sqrtf(t));
    return fminf(31.0f, floorf(32.0f * v));
}

// FP64 squared distance, evaluated as ((dx*dx + dy*dy) + dz*dz) without
// contraction, nearest image when periodic; this is the parity rule's metric.
__device__ __forceinline__ double d2_exact(const double *__restrict__ p64, int32_t a, int32_t b,
                                           bool periodic, double box) {
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        double d = __dsub_rn(p64[(int64_t)b * 3 + c], p64[(int64_t)a * 3 + c]);
        if (periodic && fabs(d) > 0.5 * box) d = -copysign(__dsub_rn(box, fabs(d)), d);
        s = __dadd_rn(s, __dmul_rn(d, d));
    }
    return s;
}

// Bitonic sort of one (key, tie) pair per lane, ascending.
template <class K>
__device__ __forceinline__ void warp_sort_pairs(K &key, int32_t &tie) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            K ok = __shfl_xor_sync(0xffffffffu, key, stride);
            int32_t ot = __shfl_xor_sync(0xffffffffu, tie, stride);
            const bool up = ((lane & size) == 0);
            const bool lower = ((lane & stride) == 0);
            const bool other_less = (ok < key) || (ok == key && ot < tie);
            // lower lane keeps the smaller when ascending
            const bool take = (lower == up) ? other_less : !other_less && !(ok == key && ot == tie);
            if (take) {
                key = ok;
                tie = ot;
            }
        }
    }
}

// Box index c (< 128) -> (ix, iy, iz) without integer division: the float
// quotients are exact enough for these small operands.
__device__ __forceinline__ void box_index(int c, float inv_nx, float inv_nxy, const int cnum[3], int &ix, int &iy,
                                          int &iz) {
    iz = (int)(((float)c + 0.5f) * inv_nxy);
    const int r = c - iz * cnum[0] * cnum[1];
    iy = (int)(((float)r + 0.5f) * inv_nx);
    ix = r - iy * cnum[0];
}

// Per-warp shared memory (KPL = neighbours per lane: k <= 32 KPL).
template <int KPL>
struct KnnSmem {
    static constexpr int kCap = KPL == 1 ? 224 : (KPL == 2 ? 320 : 448);  // candidate buffer
    float d[kCap];                  // candidate d^2
    int32_t i[kCap];                // candidate slot
    int32_t hist[32];
    float sel[32 * KPL];            // d^2 of the selected neighbours
    uint32_t ca[kList], cb[kList];  // cached box: cell ranges by box index
    uint32_t pa[kList], pb[kList];  // scan list of the current query
    uint64_t pc[kList];             // scan-list cell: level | x << 5 | y << 24 | z << 43
    uint32_t off[kList + 1];        // scan-list prefix offsets
};

struct WarpStats {
    int64_t cand = 0, retry = 0, band = 0, unres = 0, newton = 0, heavy = 0;
    int64_t reason[3] = {0, 0, 0};
    int64_t phase[6] = {0, 0, 0, 0, 0, 0};
};

// Optional per-phase cycle counters (build with -DMG_KNN_PROFILE): stats[10..13]
// accumulate clock64() cycles of box lookup, list building, scan and selection,
// summed over warps; stats[14] the cycles of the slowest warp, stats[15] the
// number of scans over more than 8192 particles done by one warp.
#ifdef MG_KNN_PROFILE
#define KNN_TICK(var) const long long var = clock64()
#define KNN_PHASE(i, t0, t1) st.phase[i] += (t1) - (t0)
#else
#define KNN_TICK(var)
#define KNN_PHASE(i, t0, t1)
#endif

// Rare path: more than 32 candidates share the histogram bucket of the k-th
// neighbour (heavy exact or near ties).  Takes the r smallest one at a time.
// Returns the k-th squared distance.
template <class SM>
__device__ __noinline__ float select_boundary_slow(SM &S, int cnt, float invR2, int dim, int b_star, int c_lo,
                                                   int r, int32_t *row) {
    const int lane = threadIdx.x & 31;
    float T = 0.0f;
    for (int rep = 0; rep < r; ++rep) {
        float best = FLT_MAX;
        int32_t bslot = INT_MAX;
        int bidx = -1;
        for (int e = lane; e < cnt; e += 32) {
            if ((int)bucket_of(S.d[e] * invR2, dim) != b_star || S.i[e] < 0) continue;
            if (S.d[e] < best || (S.d[e] == best && S.i[e] < bslot)) {
                best = S.d[e];
                bslot = S.i[e];
                bidx = e;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int32_t os = __shfl_xor_sync(0xffffffffu, bslot, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
            if (ob < best || (ob == best && os < bslot)) {
                best = ob;
                bslot = os;
                bidx = oi;
            }
        }
        if (lane == 0) {
            row[c_lo + rep] = bslot;
            S.sel[c_lo + rep] = best;
            S.i[bidx] = -1 - bslot;  // mark taken
        }
        __syncwarp();
        T = best;
    }
    for (int e = lane; e < cnt; e += 32)
        if (S.i[e] < 0) S.i[e] = -1 - S.i[e];
    __syncwarp();
    return T;
}

// Absolute half-width added to the FP64 re-decision band around the k-th
// squared distance T.  FP32 d^2 from the hi/lo positions differs from the
// FP64 d^2 by up to ~2^-23 of itself, which the relative band (kBandEps)
// covers, plus 2 sqrt(T) dd, with dd ~3e-14 |x| the separation's share of the
// positions' hi/lo representation and of the low parts' rounding (2^-46 |x|
// per axis, over three axes).  That term decides for pairs closer than ~1e-9
// of their coordinates (a tight clump far from the frame centre).  xmag: the
// query's largest coordinate magnitude (or the box side, if larger).
__device__ __forceinline__ float band_abs(float T, float xmag) {
    const float dd = 3e-14f * xmag;
    return 2.0f * sqrtf(T) * dd + dd * dd;
}
__device__ __forceinline__ float query_mag(const float4 *__restrict__ hi, int32_t p, bool periodic, float box_hi) {
    const float4 h = hi[p];
    const float m = fmaxf(fabsf(h.x), fmaxf(fabsf(h.y), fabsf(h.z)));
    return periodic ? fmaxf(m, box_hi) : m;
}

// Rare path: several candidates lie within 1e-5 (relative, in d^2, widened by
// band_abs) of the k-th distance T.  Those are re-ranked by exact FP64 d^2 and then particle index;
// everything below the band is kept.  Rewrites the whole row.  Returns false
// if the band holds more than 32 candidates (flagged unresolved).
template <class SM>
__device__ __noinline__ bool resolve_band_fp64(SM &S, int cnt, float T, float wabs, int k, int32_t p, int32_t *row,
                                               const double *__restrict__ pos64, const int32_t *__restrict__ order,
                                               bool periodic, double box) {
    const int lane = threadIdx.x & 31;
    const float lo_band = T * (1.0f - kBandEps) - wabs, hi_band = T * (1.0f + kBandEps) + wabs;
    int nb = 0, nsure = 0;
    for (int e0 = 0; e0 < cnt; e0 += 32) {
        const int e = e0 + lane;
        const bool inb = e < cnt && S.d[e] >= lo_band && S.d[e] <= hi_band;
        const bool sure = e < cnt && S.d[e] < lo_band;
        const unsigned mb = __ballot_sync(0xffffffffu, inb);
        const unsigned ms = __ballot_sync(0xffffffffu, sure);
        if (inb) {
            const int pos = nb + __popc(mb & ((1u << lane) - 1u));
            if (pos < 32) S.pb[pos] = (uint32_t)S.i[e];
        }
        if (sure) {
            const int pos = nsure + __popc(ms & ((1u << lane) - 1u));
            row[pos] = S.i[e];
            S.sel[pos] = S.d[e];
        }
        nb += __popc(mb);
        nsure += __popc(ms);
    }
    __syncwarp();
    const int need = k - nsure;
    double key = DBL_MAX;
    int32_t tie = INT_MAX, carry = p;
    if (lane < min(nb, 32)) {
        carry = (int32_t)S.pb[lane];
        key = d2_exact(pos64, p, carry, periodic, box);
        tie = order[carry];
    }
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            const double okey = __shfl_xor_sync(0xffffffffu, key, stride);
            const int32_t otie = __shfl_xor_sync(0xffffffffu, tie, stride);
            const int32_t ocar = __shfl_xor_sync(0xffffffffu, carry, stride);
            const bool up = ((lane & size) == 0);
            const bool lower = ((lane & stride) == 0);
            const bool other_less = (okey < key) || (okey == key && otie < tie);
            const bool same = (okey == key && otie == tie);
            if ((lower == up) ? other_less : (!other_less && !same)) {
                key = okey;
                tie = otie;
                carry = ocar;
            }
        }
    }
    if (lane < need) {
        row[nsure + lane] = carry;
        S.sel[nsure + lane] = (float)key;
    }
    __syncwarp();
    return !(nb > 32 || need > 32 || need > nb);
}

// FP32 squared distance from the query (h0, l0) to slot t; one expression for
// every path so that all of them see the same value.
__device__ __forceinline__ float cand_d2p(const float4 *__restrict__ hi, const float4 *__restrict__ lo, bool periodic,
                                         float box_hi, float box_lo, const float4 &h0, const float4 &l0, uint32_t t) {
    const float4 hb = hi[t], lb = lo[t];
    const float3 sv = periodic ? sep_hilo_periodic(h0, l0, hb, lb, box_hi, box_lo) : sep_hilo(h0, l0, hb, lb);
    return __fmaf_rn(sv.z, sv.z, __fmaf_rn(sv.y, sv.y, __fmul_rn(sv.x, sv.x)));
}
__device__ __forceinline__ float cand_d2(const KnnArgs &a, const float4 &h0, const float4 &l0, uint32_t t) {
    return cand_d2p(a.hi, a.lo, a.periodic, a.box_hi, a.box_lo, h0, l0, t);
}

// Scan-list candidate g -> slot, for a 32-wide chunk starting at g0: the
// boundaries of entries that start inside the chunk are OR-reduced into a bit
// mask and each lane counts those at or below it.  j0: entry holding g0 (updated
// to the entry holding g0 + 32).
template <class SM>
__device__ __forceinline__ uint32_t chunk_slot(const SM &S, int nlist, int total, int g0, int &j0, int lane) {
    const int bidx = j0 + 1 + lane;
    const uint32_t bnd = bidx <= nlist ? S.off[bidx] : 0xffffffffu;
    const uint32_t rel = bnd - (uint32_t)g0;
    const uint32_t bit = (bnd != 0xffffffffu && rel < 32u) ? (1u << rel) : 0u;
    const uint32_t mask = __reduce_or_sync(0xffffffffu, bit);
    const int j = j0 + __popc(mask & ((2u << lane) - 1u));
    const uint32_t t = g0 + lane < total ? S.pa[j] + (uint32_t)(g0 + lane - (int)S.off[j]) : 0u;
    j0 = __shfl_sync(0xffffffffu, j, 31);
    if (j0 + 1 <= nlist && (int)S.off[j0 + 1] == g0 + 32) ++j0;
    return t;
}

// Rare path (out of line, so that it stays out of the scan loop's instruction
// stream): the buffer overflowed during the scan, whose in-radius candidates
// beyond the buffer were binned into S.hist (32 buckets of (d/R)^dim).  Narrows
// the bucket of the k-th neighbour with up to two re-scans of 32 sub-buckets
// each.  Returns the upper edge v_hi (in (d/R)^dim) of the narrowest bucket
// found whose cumulative count reaches k.
template <int DIM, class SM>
__device__ __noinline__ float overflow_window(SM &S, const float4 *__restrict__ hi, const float4 *__restrict__ lo,
                                              bool periodic, float box_hi, float box_lo, float4 h0, float4 l0,
                                              int nlist, int total, float R2, int k, int cap) {
    const int lane = threadIdx.x & 31;
    const float invR2 = 1.0f / R2;
    float v_lo = 0.0f, v_w = 1.0f / 32.0f, v_hi = 1.0f;
    int c_below = 0;
    for (int level = 0; level < 3; ++level) {
        if (level > 0) {  // re-scan, binning the current window into 32 sub-buckets
            int j0 = 0;
            for (int g0 = 0; g0 < total; g0 += 32) {
                const uint32_t t = chunk_slot(S, nlist, total, g0, j0, lane);
                if (g0 + lane < total) {
                    const float dd = cand_d2p(hi, lo, periodic, box_hi, box_lo, h0, l0, t);
                    if (dd <= R2) {
                        const float tt = dd * invR2;
                        const float v = DIM == 3 ? tt * sqrtf(tt) : (DIM == 2 ? tt : sqrtf(tt));
                        if (v >= v_lo && v < v_hi) atomicAdd(&S.hist[min(31, (int)((v - v_lo) / v_w))], 1);
                    }
                }
            }
            __syncwarp();
        }
        // locate the sub-bucket holding the k-th and narrow the window
        const int hc = S.hist[lane];
        const int cum = warp_incl_scan(hc) + c_below;
        const int bk = __ffs(__ballot_sync(0xffffffffu, cum >= k)) - 1;
        const int cum_bk = __shfl_sync(0xffffffffu, cum, max(bk, 0));
        const int hc_bk = __shfl_sync(0xffffffffu, hc, max(bk, 0));
        if (bk < 0) break;  // numerical edge: keep the window
        v_hi = v_lo + (float)(bk + 1) * v_w;
        if (cum_bk <= cap) break;
        c_below = cum_bk - hc_bk;
        v_lo = v_lo + (float)bk * v_w;
        v_w = v_w / 32.0f;
        __syncwarp();
        S.hist[lane] = 0;
        __syncwarp();
    }
    return v_hi;
}

// Rare path: the buffer has just overflowed; bin the buffered candidates
// (kept out of the scan loop's instruction stream unless MG_KNN_LAZY_INLINE).
#ifdef MG_KNN_LAZY_INLINE
#define KNN_LAZY_INLINE __forceinline__
#else
#define KNN_LAZY_INLINE __noinline__
#endif
template <int DIM, class SM>
__device__ KNN_LAZY_INLINE void lazy_hist_init(SM &S, float invR2) {
    const int lane = threadIdx.x & 31;
    S.hist[lane] = 0;
    __syncwarp();
    for (int e = lane; e < SM::kCap; e += 32) atomicAdd(&S.hist[(int)bucket_of(S.d[e] * invR2, DIM)], 1);
    __syncwarp();
}

// Rare path (out of line): entries of the scan-list chunk starting at i0 that
// hold more than kSplit particles and straddle the sphere are replaced by their
// non-empty children that meet it (open 3-D boxes; children of a level-l cell
// are consecutive Morton codes, so 7 binary searches inside the parent's range
// give all 8 ranges).  Returns the new list length.
template <class SM>
__device__ __noinline__ int split_chunk(SM &S, int i0, int nlist, float ux0, float uy0, float uz0, float Rs, float rc,
                                        int L, const uint64_t *__restrict__ keys) {
    const int lane = threadIdx.x & 31;
    const int i = i0 + lane;
    bool split = false;
    if (i < nlist && S.pb[i] - S.pa[i] > (uint32_t)kSplit) {
        const uint64_t pc = S.pc[i];
        const int lv = (int)(pc & 31u);
        if (lv < kMaxLevel) {
            const float f = exp2f((float)(lv - L));
            const float x0 = (float)((pc >> 5) & 0x7ffffu), y0 = (float)((pc >> 24) & 0x7ffffu),
                        z0 = (float)((pc >> 43) & 0x7ffffu);
            const float ux = ux0 * f, uy = uy0 * f, uz = uz0 * f;
            const float fx = fmaxf(fabsf(ux - x0), fabsf(ux - x0 - 1.0f));
            const float fy = fmaxf(fabsf(uy - y0), fabsf(uy - y0 - 1.0f));
            const float fz = fmaxf(fabsf(uz - z0), fabsf(uz - z0 - 1.0f));
            const float rin = Rs * f * (1.0f - 1e-5f);
            split = fx * fx + fy * fy + fz * fz > rin * rin;  // not entirely inside
        }
    }
    unsigned sm = __ballot_sync(0xffffffffu, split);
    while (sm) {
        const int j = __ffs(sm) - 1;
        sm &= sm - 1;
        const int idx = i0 + j;
        const uint32_t A = S.pa[idx], B = S.pb[idx];
        const uint64_t pc = S.pc[idx];
        const int lv = (int)(pc & 31u) + 1;
        const uint32_t x0 = (uint32_t)((pc >> 5) & 0x7ffffu) * 2u, y0 = (uint32_t)((pc >> 24) & 0x7ffffu) * 2u,
                       z0 = (uint32_t)((pc >> 43) & 0x7ffffu) * 2u;
        const int ch = lane & 7;
        const uint32_t cx = x0 + (ch & 1), cy = y0 + ((ch >> 1) & 1), cz = z0 + (ch >> 2);
        const uint64_t code = morton3(cx, cy, cz);
        uint32_t lo = A;
        if (lane >= 1 && lane < 8) lo = lower_bound_prefix(keys, A, B, code, 3 * (kKeyBits - lv));
        uint32_t hi = __shfl_down_sync(0xffffffffu, lo, 1);
        if (ch == 7) hi = B;
        bool keep = false;
        if (lane < 8 && hi > lo) {
            const float f = exp2f((float)(lv - L));
            const float ux = ux0 * f, uy = uy0 * f, uz = uz0 * f, rr = rc * f;
            const float dx = fmaxf(0.0f, fmaxf((float)cx - ux, ux - (float)(cx + 1)));
            const float dy = fmaxf(0.0f, fmaxf((float)cy - uy, uy - (float)(cy + 1)));
            const float dz = fmaxf(0.0f, fmaxf((float)cz - uz, uz - (float)(cz + 1)));
            keep = dx * dx + dy * dy + dz * dz <= rr * rr;
        }
        const unsigned km = __ballot_sync(0xffffffffu, keep);
        if (nlist + __popc(km) <= kList) {
            const int pos = nlist + __popc(km & ((1u << lane) - 1u));
            if (keep) {
                S.pa[pos] = lo;
                S.pb[pos] = hi;
                S.pc[pos] = (uint64_t)lv | ((uint64_t)cx << 5) | ((uint64_t)cy << 24) | ((uint64_t)cz << 43);
            }
            nlist += __popc(km);
            if (lane == 0) S.pb[idx] = S.pa[idx];  // parent replaced by its children
        }
        __syncwarp();
    }
    return nlist;
}

// The k smallest of the cnt buffered candidates (all with d^2 <= R^2) by a
// 32-bucket histogram in (d/R)^dim: buckets below the k-th one are taken
// whole, the k-th bucket is sorted.  Writes the row and S.sel; returns the
// k-th squared distance T.
template <int DIM, class SM>
__device__ KNN_SELECT_INLINE float select_k(SM &S, int cnt, float invR2, int k, int32_t *row) {
    const int lane = threadIdx.x & 31;
    float T;
    S.hist[lane] = 0;
    __syncwarp();
    KNN_LOOP_HINT
    for (int e = lane; e < cnt; e += 32) atomicAdd(&S.hist[(int)bucket_of(S.d[e] * invR2, DIM)], 1);
    __syncwarp();
    const int hcount = S.hist[lane];
    const int cum = warp_incl_scan(hcount);
    const int b_star = __ffs(__ballot_sync(0xffffffffu, cum >= k)) - 1;
    const int cum_b = __shfl_sync(0xffffffffu, cum, b_star);
    const int m_b = __shfl_sync(0xffffffffu, hcount, b_star);
    const int c_lo = cum_b - m_b;
    const int r = k - c_lo;
    int out = 0, nb = 0;
    KNN_LOOP_HINT
    for (int e0 = 0; e0 < cnt; e0 += 32) {
        const int e = e0 + lane;
        const float v = e < cnt ? S.d[e] : FLT_MAX;
        const int bk = e < cnt ? (int)bucket_of(v * invR2, DIM) : 99;
        const bool sure = bk < b_star;
        const unsigned ms = __ballot_sync(0xffffffffu, sure);
        if (sure) {
            const int pos = out + __popc(ms & ((1u << lane) - 1u));
            row[pos] = S.i[e];
            S.sel[pos] = v;
        }
        out += __popc(ms);
        const bool bnd = bk == b_star;
        const unsigned mb = __ballot_sync(0xffffffffu, bnd);
        if (bnd && m_b <= 32) {
            const int pos = nb + __popc(mb & ((1u << lane) - 1u));
            S.pa[pos] = __float_as_uint(v);
            S.pb[pos] = (uint32_t)S.i[e];
        }
        nb += __popc(mb);
    }
    __syncwarp();
    if (m_b <= 32) {
        float key = lane < m_b ? __uint_as_float(S.pa[lane]) : FLT_MAX;
        int32_t tie = lane < m_b ? (int32_t)S.pb[lane] : INT_MAX;
        warp_sort_pairs(key, tie);
        if (lane < r) {
            row[c_lo + lane] = tie;
            S.sel[c_lo + lane] = key;
        }
        T = __shfl_sync(0xffffffffu, key, r - 1);
    } else {
        T = select_boundary_slow(S, cnt, invR2, DIM, b_star, c_lo, r, row);
    }
    __syncwarp();
    return T;
}

// After select_k (band inside the radius): candidates within 1e-5 of T are
// re-decided in FP64, then the selected d^2 are stored for the h solve.  A band
// of more than 32 flags the query unresolved.
template <class SM>
__device__ KNN_SELECT_INLINE void finish_row(SM &S, int cnt, float T, int k, int32_t p, int32_t qi, const KnnArgs &a,
                                             double side, WarpStats &st) {
    const int lane = threadIdx.x & 31;
    int32_t *row = a.ngb + (int64_t)qi * k;
    const float wabs = band_abs(T, query_mag(a.hi, p, a.periodic, a.box_hi));
    const float lo_band = T * (1.0f - kBandEps) - wabs, hi_band = T * (1.0f + kBandEps) + wabs;
    int nband = 0;
    KNN_LOOP_HINT
    for (int e0 = 0; e0 < cnt; e0 += 32) {
        const int e = e0 + lane;
        const bool inb = e < cnt && S.d[e] >= lo_band && S.d[e] <= hi_band;
        nband += __popc(__ballot_sync(0xffffffffu, inb));
    }
    if (nband > 1) {
        st.band += 1;
        const bool ok = resolve_band_fp64(S, cnt, T, wabs, k, p, row, a.pos64, a.order, a.periodic, side);
        if (!ok) {
            if (lane == 0) {
                atomicOr(a.qstatus + qi, MG_Q_UNRESOLVED);
                a.hsml[qi] = -(float)(4000000);
            }
            st.unres += 1;
            return;
        }
        if (lane == 0) atomicOr(a.qstatus + qi, MG_Q_BAND_FP64);
    }
}

template <int DIM, int KPL>
__device__ __forceinline__ void knn_warp_pass(const KnnArgs &a, unsigned char *knn_smem) {
    using SM = KnnSmem<KPL>;
    constexpr int kKnnCap = SM::kCap;
    SM &S = reinterpret_cast<SM *>(knn_smem)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t gwarp = (int64_t)blockIdx.x * kKnnWarps + wib;
    const int64_t nwarps = (int64_t)gridDim.x * kKnnWarps;
    // the queue, radii and brackets of this pass were written by other blocks
    // of an earlier pass (of the same launch, for the cooperative passes): read
    // at L2 (__ldcg), never from a stale L1 line
    const int64_t count = a.qin ? (int64_t)__ldcg(a.qin_count) : a.nq;
    const Frame fr = load_frame(a.frame);
    const float side = (float)fr.side;
    const float half_side = 0.5f * side;
    const int k = a.k;

    WarpStats st;
#ifdef MG_KNN_PROFILE
    const long long t_warp0 = clock64();
#endif
    int32_t my_retry = -1;  // lane i holds the i-th pending retry of this warp
    int n_retry = 0;

    // Each warp takes runs of MG_KNN_WCHUNK queries dealt to the warps in
    // turn (the slow regions of the queue spread over the warps), or with 0
    // one contiguous run; a warp reuses the cell-box ranges of its previous
    // query when the next one needs the same box (consecutive queries are
    // neighbours in Morton order).
    int cL = -1, cmin_c[3] = {0, 0, 0}, cnum_c[3] = {0, 0, 0};  // cached box
#if MG_KNN_WCHUNK > 0
    for (int64_t c0 = gwarp * MG_KNN_WCHUNK; c0 < count; c0 += nwarps * MG_KNN_WCHUNK)
    for (int64_t item = c0, item1 = min(count, c0 + (int64_t)MG_KNN_WCHUNK); item < item1; ++item) {
#else
    const int64_t per_warp = (count + nwarps - 1) / nwarps;
    const int64_t item0 = gwarp * per_warp;
    const int64_t item1 = min(count, item0 + per_warp);
    for (int64_t item = item0; item < item1; ++item) {
#endif
        KNN_TICK(t_a);
        const int32_t qi = a.qin ? __ldcg(a.qin + item) : (int32_t)item;
        const int32_t p = a.queries ? a.queries[qi] : qi;
        float R = a.qin ? __ldcg(a.radius + qi) : a.seed_h[qi] * a.radius_factor;
        // a negative queued radius was set by the block-wide path from a histogram
        // of the distances: it holds at least k and at most a buffer, so it is
        // scanned by this warp whatever the size of its scan list
        const bool cert = a.qin && R < 0.0f;
        R = fabsf(R);
        if (!(R > 0.0f) || !isfinite(R)) R = side * 1e-3f;
        float rlo = a.qin ? __ldcg(a.rlo + qi) : 0.0f, rhi = a.qin ? __ldcg(a.rhi + qi) : 0.0f;
        const float4 h0 = a.hi[p], l0 = a.lo[p];

        // ---- level and cell box ------------------------------------------
        // level_bias 1 allows R up to two cell sides, so with the rounding
        // margin of rc a box can reach 6 cells per axis; a box over kList
        // cells (the per-warp cache) is redone one level coarser (<= 4 per axis)
        int L = (int)floorf(log2f(side / R)) + a.level_bias;
        L = max(0, min(kMaxLevel, L));
        float cells_per_side, scale, u[3], rc;
        int cmin[3], cnum[3], ncell;
        bool full[3];  // periodic axis covered entirely: no distance test
        for (;;) {
            cells_per_side = (float)(1u << L);
            scale = cells_per_side / side;
            u[0] = ((h0.x + half_side) + l0.x) * scale;
            u[1] = ((h0.y + half_side) + l0.y) * scale;
            u[2] = ((h0.z + half_side) + l0.z) * scale;
            rc = R * scale * (1.0f + 1e-5f) + 1e-3f + cells_per_side * 2.4e-7f;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                full[d] = false;
                if (d >= DIM) {
                    cmin[d] = 0;
                    cnum[d] = 1;
                    continue;
                }
                int lo_c = (int)floorf(u[d] - rc), hi_c = (int)floorf(u[d] + rc);
                if (a.periodic) {
                    if (hi_c - lo_c + 1 >= (int)cells_per_side) {
                        lo_c = 0;
                        hi_c = (int)cells_per_side - 1;
                        full[d] = true;
                    }
                } else {
                    lo_c = max(lo_c, 0);
                    hi_c = min(hi_c, (int)cells_per_side - 1);
                }
                cmin[d] = lo_c;
                cnum[d] = max(0, hi_c - lo_c + 1);
            }
            ncell = cnum[0] * cnum[1] * cnum[2];
            if (ncell <= kList || L == 0) break;
            --L;
        }
        const float R2 = R * R;
        const float inv_nx = 1.0f / (float)max(cnum[0], 1), inv_nxy = 1.0f / (float)max(cnum[0] * cnum[1], 1);

        // ---- cell ranges: look up the box unless it is the cached one --------
        const bool same_box = (L == cL) && cmin[0] == cmin_c[0] && cmin[1] == cmin_c[1] && cmin[2] == cmin_c[2] &&
                              cnum[0] == cnum_c[0] && cnum[1] == cnum_c[1] && cnum[2] == cnum_c[2];
        if (!same_box) {
            // Cells that the previous box (same level) also held are copied from
            // the cache instead of looked up again (consecutive queries' boxes
            // are mostly shifted copies of each other); the new ranges are staged
            // in the scan-list arrays, free at this point, then moved.
            const bool shift_ok = L == cL;
            KNN_LOOP_HINT
            for (int cb = 0; cb < ncell; cb += 32) {
                const int c = cb + lane;
                if (c < ncell) {
                    int ix, iy, iz;
                    box_index(c, inv_nx, inv_nxy, cnum, ix, iy, iz);
                    int gx = cmin[0] + ix, gy = cmin[1] + iy, gz = cmin[2] + iz;
                    const int ox = gx - cmin_c[0], oy = gy - cmin_c[1], oz = gz - cmin_c[2];
                    uint32_t ca, cbnd;
                    if (shift_ok && ox >= 0 && ox < cnum_c[0] && oy >= 0 && oy < cnum_c[1] && oz >= 0 &&
                        oz < cnum_c[2]) {
                        const int oc = ox + cnum_c[0] * (oy + cnum_c[1] * oz);
                        ca = S.ca[oc];
                        cbnd = S.cb[oc];
                    } else {
                        const int M = (int)cells_per_side;
                        if (a.periodic) {
                            gx = ((gx % M) + M) % M;
                            gy = ((gy % M) + M) % M;
                            gz = ((gz % M) + M) % M;
                        }
                        if (DIM < 3) gz = 0;
                        if (DIM < 2) gy = 0;
                        cell_range(a.ci, L, (uint32_t)gx, (uint32_t)gy, (uint32_t)gz, ca, cbnd);
                    }
                    S.pa[c] = ca;
                    S.pb[c] = cbnd;
                }
            }
            __syncwarp();
            KNN_LOOP_HINT
            for (int c = lane; c < ncell; c += 32) {
                S.ca[c] = S.pa[c];
                S.cb[c] = S.pb[c];
            }
            cL = L;
            for (int d = 0; d < 3; ++d) {
                cmin_c[d] = cmin[d];
                cnum_c[d] = cnum[d];
            }
            __syncwarp();
        }
        KNN_TICK(t_b);
        KNN_PHASE(0, t_a, t_b);
        // prune to the non-empty cells that meet this query's sphere
        int nlist = 0;
        KNN_LOOP_HINT
        for (int cb = 0; cb < ncell; cb += 32) {
            const int c = cb + lane;
            bool use = false;
            uint32_t ca = 0, cbnd = 0;
            int gx = 0, gy = 0, gz = 0;
            if (c < ncell) {
                ca = S.ca[c];
                cbnd = S.cb[c];
                int ix, iy, iz;
                box_index(c, inv_nx, inv_nxy, cnum, ix, iy, iz);
                gx = cmin[0] + ix;
                gy = cmin[1] + iy;
                gz = cmin[2] + iz;
                float dx = full[0] ? 0.0f : fmaxf(0.0f, fmaxf((float)gx - u[0], u[0] - (float)(gx + 1)));
                float dy = full[1] ? 0.0f : fmaxf(0.0f, fmaxf((float)gy - u[1], u[1] - (float)(gy + 1)));
                float dz = full[2] ? 0.0f : fmaxf(0.0f, fmaxf((float)gz - u[2], u[2] - (float)(gz + 1)));
                if (DIM < 3) dz = 0.0f;
                if (DIM < 2) dy = 0.0f;
                use = cbnd > ca && dx * dx + dy * dy + dz * dz <= rc * rc;
            }
            const unsigned m = __ballot_sync(0xffffffffu, use);
            const int pos = nlist + __popc(m & ((1u << lane) - 1u));
            if (use) {
                S.pa[pos] = ca;
                S.pb[pos] = cbnd;
                S.pc[pos] = (uint64_t)L | ((uint64_t)(uint32_t)gx << 5) | ((uint64_t)(uint32_t)gy << 24) |
                            ((uint64_t)(uint32_t)gz << 43);
            }
            nlist += __popc(m);
        }
        __syncwarp();
        // Split big cells that straddle the sphere into their 8 children: near a
        // dense clump or core the coarse cells of a sparse query would otherwise
        // put far more particles into the scan than the sphere holds.
        if (DIM == 3 && !a.periodic) {
            KNN_LOOP_HINT
            for (int i0 = 0; i0 < nlist; i0 += 32) {
                const int i = i0 + lane;
                const bool big = i < nlist && S.pb[i] - S.pa[i] > (uint32_t)kSplit;
                if (__any_sync(0xffffffffu, big)) nlist = split_chunk(S, i0, nlist, u[0], u[1], u[2], R * scale, rc, L, a.keys);
            }
        }
        // drop emptied entries and form prefix offsets (entries strictly non-empty)
        {
            int w = 0, total = 0;
            KNN_LOOP_HINT
            for (int i0 = 0; i0 < nlist; i0 += 32) {
                const int i = i0 + lane;
                const uint32_t ra = i < nlist ? S.pa[i] : 0u, rb = i < nlist ? S.pb[i] : 0u;
                const int n_i = (int)(rb - ra);
                __syncwarp();
                const unsigned m = __ballot_sync(0xffffffffu, n_i > 0);
                const int inc = warp_incl_scan(n_i);
                if (n_i > 0) {
                    const int pos = w + __popc(m & ((1u << lane) - 1u));
                    S.pa[pos] = ra;
                    S.pb[pos] = rb;
                    S.off[pos] = (uint32_t)(total + inc - n_i);
                }
                w += __popc(m);
                total += __shfl_sync(0xffffffffu, inc, 31);
            }
            nlist = w;
            if (lane == 0) S.off[nlist] = (uint32_t)total;
            __syncwarp();
#ifdef MG_KNN_DEBUG
            // scan-list entries must be disjoint slot ranges
            for (int e = lane; e < nlist; e += 32) {
                const uint32_t ea = S.pa[e], eb = S.pa[e] + (S.off[e + 1] - S.off[e]);
                for (int j = 0; j < nlist; ++j) {
                    const uint32_t ja = S.pa[j], jb = S.pa[j] + (S.off[j + 1] - S.off[j]);
                    if (j != e && ea < jb && ja < eb) {
                        atomicAdd((unsigned long long *)&a.stats[15], 1ull);
                        atomicMax((unsigned long long *)&a.stats[14], (unsigned long long)qi);
                    }
                }
            }
            __syncwarp();
#endif
            st.cand += total;
            KNN_TICK(t_c);
            KNN_PHASE(1, t_b, t_c);
            // ---- gather candidates with d^2 <= R^2 -------------------------
            // mode 0 fills the buffer; modes 1..3 (only after an overflow) scan
            // again and histogram the in-radius candidates so the next radius
            // can be cut to the bucket that holds the k-th neighbour.  More than
            // kScanLimit particles in the scan list: no scan, the radius shrinks
            // by the volume ratio (bracketed).
            int cnt = 0;
            const float invR2 = 1.0f / R2;
            // (only before any radius of this query has held fewer than k:
            // after that the box is always scanned, so the search converges)
            const bool too_big = total > kScanLimit && rlo == 0.0f && !cert;
            // a long scan list goes to the block-wide path (k_knn_heavy) with
            // its list, so that one warp does not scan it several times while
            // the rest of the grid waits for it
            if (!too_big && !cert && total > kHeavy && a.heavy_cap > 0) {
                int slot = 0;
                if (lane == 0) slot = atomicAdd(a.heavy_count, 1);
                slot = __shfl_sync(0xffffffffu, slot, 0);
                if (slot < a.heavy_cap) {
                    int32_t *item = a.heavy + (int64_t)slot * kHeavyItem;
                    if (lane == 0) {
                        item[0] = qi;
                        item[1] = nlist;
                        a.radius[qi] = R;
                        a.rlo[qi] = rlo;
                        a.rhi[qi] = rhi;
                    }
                    for (int e = lane; e < nlist; e += 32) item[2 + e] = (int32_t)S.pa[e];
                    for (int e = lane; e <= nlist; e += 32) item[2 + kList + e] = (int32_t)S.off[e];
                    st.heavy += 1;
                    __syncwarp();
                    continue;
                }
            }
            float v_hi = 1.0f;
            if (!too_big) {
                int j0 = 0;
                KNN_LOOP_HINT
                for (int g0 = 0; g0 < total; g0 += 32) {
                    const uint32_t t = chunk_slot(S, nlist, total, g0, j0, lane);
                    const float dd = g0 + lane < total ? cand_d2(a, h0, l0, t) : FLT_MAX;
                    const bool in = dd <= R2;
                    const unsigned m = __ballot_sync(0xffffffffu, in);
                    const int pos = cnt + __popc(m & ((1u << lane) - 1u));
                    if (in && pos < kKnnCap) {
                        S.d[pos] = dd;
                        S.i[pos] = (int32_t)t;
                    }
                    const int before = cnt;
                    cnt += __popc(m);
                    // Lazy histogram: the first time the buffer overflows, the
                    // buffered candidates are binned; from then on every new
                    // in-radius candidate is binned directly, so an overflow
                    // usually needs no second scan.
                    if (before <= kKnnCap && cnt > kKnnCap) lazy_hist_init<DIM>(S, invR2);
                    if (cnt > kKnnCap && in && pos >= kKnnCap) atomicAdd(&S.hist[(int)bucket_of(dd * invR2, DIM)], 1);
                }
                __syncwarp();
                if (cnt > kKnnCap)
                    v_hi = overflow_window<DIM>(S, a.hi, a.lo, a.periodic, a.box_hi, a.box_lo, h0, l0, nlist, total, R2,
                                                k, kKnnCap);
            }

            KNN_TICK(t_d);
            KNN_PHASE(2, t_c, t_d);
#ifdef MG_KNN_PROFILE
            if (total > 8192) st.phase[5] += 1;  // big single-warp scans
#endif
            // ---- radius updates (bracketed) ------------------------------------
            // rlo: largest radius seen holding fewer than k; rhi: smallest radius
            // seen holding more than the buffer (so at least k).  Growth is a
            // geometric guess capped by rhi (geometric mean once both are known);
            // an overflow cuts the radius to the histogram bucket holding the k-th
            // neighbour, which holds at least k by construction.
            float Rnew = -1.0f;
            int reason = 0;
            if (too_big) {
                Rnew = R * fmaxf(0.25f, powf(0.5f * kKnnCap / (float)total, 1.0f / DIM));
                reason = 2;
            } else if (cnt < k) {
                rlo = fmaxf(rlo, R);
                const float g = 1.25f * powf((float)k / (float)max(cnt, 1), 1.0f / DIM);
                Rnew = R * fminf(fmaxf(g, 1.25f), 4.0f);
                if (rhi > 0.0f && Rnew >= rhi) Rnew = sqrtf(rlo * rhi);
                reason = 1;
            } else if (cnt > kKnnCap) {
                rhi = (rhi > 0.0f) ? fminf(rhi, R) : R;
                Rnew = R * (DIM == 3 ? cbrtf(v_hi) : (DIM == 2 ? sqrtf(v_hi) : v_hi)) * 1.00001f;
                if (Rnew >= R) Rnew = R * 0.999f;
                reason = 2;
            }

            // ---- select the k smallest: bucket histogram ------------------------
            float T = 0.0f;
            int32_t *row = a.ngb + (int64_t)qi * k;
            if (Rnew < 0.0f) {
                T = select_k<DIM>(S, cnt, invR2, k, row);
                // the band around T must lie inside the searched radius
                const float wabs = band_abs(T, query_mag(a.hi, p, a.periodic, a.box_hi));
                if (T * (1.0f + kBandEps) + 2.0f * wabs > R2) {
                    Rnew = sqrtf(T * (1.0f + 2.0f * kBandEps) + 4.0f * wabs) * 1.0001f;
                    reason = 3;
                }
            }

            KNN_TICK(t_e);
            KNN_PHASE(3, t_d, t_e);
            if (Rnew > 0.0f) {
                st.reason[reason - 1] += 1;
                if (a.last_pass) {
                    if (lane == 0) {
                        atomicOr(a.qstatus + qi, MG_Q_UNRESOLVED);
                        // diagnostics for the caller: last radius and candidate count
                        a.radius[qi] = R;
                        a.hsml[qi] = -(float)((too_big ? total : cnt) + 1000000 * reason);
                    }
                    st.unres += 1;
                } else {
                    if (lane == 0) {
                        a.radius[qi] = Rnew;
                        a.rlo[qi] = rlo;
                        a.rhi[qi] = rhi;
                    }
                    if (lane == n_retry) my_retry = qi;
                    ++n_retry;
                    st.retry += 1;
                    if (n_retry == 32) {
                        int base = 0;
                        if (lane == 0) base = atomicAdd(a.qout_count, 32);
                        base = __shfl_sync(0xffffffffu, base, 0);
                        a.qout[base + lane] = my_retry;
                        n_retry = 0;
                    }
                }
                continue;
            }

            finish_row(S, cnt, T, k, p, qi, a, fr.side, st);
        }
    }

    // flush pending retries
    if (n_retry > 0) {
        int base = 0;
        if (lane == 0) base = atomicAdd(a.qout_count, n_retry);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (lane < n_retry) a.qout[base + lane] = my_retry;
    }
    // statistics: one atomic per warp
    if (lane == 0 && a.stats) {
        if (st.cand) atomicAdd((unsigned long long *)&a.stats[1], (unsigned long long)st.cand);
        if (st.retry) atomicAdd((unsigned long long *)&a.stats[2], (unsigned long long)st.retry);
        if (st.band) atomicAdd((unsigned long long *)&a.stats[3], (unsigned long long)st.band);
        if (st.unres) atomicAdd((unsigned long long *)&a.stats[4], (unsigned long long)st.unres);
        if (st.newton) atomicAdd((unsigned long long *)&a.stats[5], (unsigned long long)st.newton);
        for (int r = 0; r < 3; ++r)
            if (st.reason[r]) atomicAdd((unsigned long long *)&a.stats[6 + r], (unsigned long long)st.reason[r]);
        if (st.heavy) atomicAdd((unsigned long long *)&a.stats[9], (unsigned long long)st.heavy);
#ifdef MG_KNN_PROFILE
        for (int r = 0; r < 6; ++r)
            if (r != 4 && st.phase[r]) atomicAdd((unsigned long long *)&a.stats[10 + r], (unsigned long long)st.phase[r]);
        atomicMax((unsigned long long *)&a.stats[14], (unsigned long long)(clock64() - t_warp0));  // slowest warp
#endif
    }
}

template <int DIM, int KPL>
__global__ __launch_bounds__(kKnnWarps * 32, kKnnMinBlocks) void k_knn_hsml(const __grid_constant__ KnnArgs a) {
    extern __shared__ __align__(16) unsigned char knn_smem[];
    knn_warp_pass<DIM, KPL>(a, knn_smem);
}


// ---- heavy queries: one block per query ------------------------------------------
// A query whose scan list holds more than kHeavy particles (a dense clump inside
// the sphere of a sparse query) is handed over with its list.  A block
// histograms the in-radius candidates in kHeavyBins bins of (d/R)^dim, narrows
// the bin holding the k-th neighbour until it and everything below it fit the
// buffer, gathers those (d^2 <= Rc^2) and warp 0 selects as the warp path does.
template <int DIM>
__device__ __forceinline__ float vol_of(float t) {  // t = d^2 / R^2
    return DIM == 3 ? t * sqrtf(t) : (DIM == 2 ? t : sqrtf(t));
}
template <int DIM>
__device__ __forceinline__ float radius_of_vol(float v) {
    return DIM == 3 ? cbrtf(v) : (DIM == 2 ? sqrtf(v) : v);
}

template <int KPL>
struct HeavySmem {
    KnnSmem<KPL> S;  // warp 0's selection buffer
    uint32_t pa[kList];
    uint32_t off[kList + 1];
    int hist[kHeavyBins];
    int wsum[kHeavyThreads / 32];
    int item, bstar, cum_prev, cum_b, cnt, total_in;
};

template <int DIM, int KPL>
__device__ __forceinline__ void knn_heavy_pass(const KnnArgs &a, HeavySmem<KPL> &H) {
    constexpr int kCap = KnnSmem<KPL>::kCap;
    static_assert(kHeavyBins == 4 * kHeavyThreads, "four bins per thread");
    static_assert(2 * kCap <= kHeavyBins, "sort scratch lives in the histogram");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int navail = min(__ldcg(a.heavy_count), a.heavy_cap);  // written by the warp path (L2 reads, as there)
    const Frame fr = load_frame(a.frame);
    const int k = a.k;
    WarpStats st;
    for (;;) {
        if (tid == 0) H.item = atomicAdd(a.heavy_next, 1);
        __syncthreads();
        const int h = H.item;
        if (h >= navail) break;
        const int32_t *item = a.heavy + (int64_t)h * kHeavyItem;
        const int32_t qi = __ldcg(item);
        const int nlist = __ldcg(item + 1);
        for (int e = tid; e < nlist; e += kHeavyThreads) H.pa[e] = (uint32_t)__ldcg(item + 2 + e);
        for (int e = tid; e <= nlist; e += kHeavyThreads) H.off[e] = (uint32_t)__ldcg(item + 2 + kList + e);
        __syncthreads();
        const int total = (int)H.off[nlist];
        const int32_t p = a.queries ? a.queries[qi] : qi;
        const float4 h0 = a.hi[p], l0 = a.lo[p];
        const float R = __ldcg(a.radius + qi);
        float rlo = __ldcg(a.rlo + qi), rhi = __ldcg(a.rhi + qi);
        const float R2 = R * R, invR2 = 1.0f / R2;
        // candidate g of the flattened list -> slot (largest entry with off <= g)
        auto slot_of = [&](int g) -> uint32_t {
            int lo = 0, hi = nlist - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if ((int)H.off[mid] <= g)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            return H.pa[lo] + (uint32_t)(g - (int)H.off[lo]);
        };

        // ---- narrow the bin of the k-th neighbour ----------------------------
        float v_lo = 0.0f, v_w = 1.0f / kHeavyBins, Rc = -1.0f;
        int c_below = 0, in_radius = -1;
        for (int lev = 0; lev < 3; ++lev) {
            for (int b = tid; b < kHeavyBins; b += kHeavyThreads) H.hist[b] = 0;
            if (tid == 0) H.bstar = -1;
            __syncthreads();
            for (int g0 = tid; g0 < total; g0 += 4 * kHeavyThreads) {
                float dd[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int g = g0 + u * kHeavyThreads;
                    dd[u] = g < total ? cand_d2(a, h0, l0, slot_of(g)) : FLT_MAX;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (dd[u] <= R2) {
                        const float v = vol_of<DIM>(dd[u] * invR2);
                        if (v >= v_lo) {
                            const float x = (v - v_lo) / v_w;  // lev 0: v <= 1, the last bin takes v == 1
                            if (x < (float)kHeavyBins)
                                atomicAdd(&H.hist[(int)x], 1);
                            else if (lev == 0)
                                atomicAdd(&H.hist[kHeavyBins - 1], 1);
                        }
                    }
                }
            }
            __syncthreads();
            {
                int c[4], sum = 0;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    c[u] = H.hist[4 * tid + u];
                    sum += c[u];
                }
                const int incl = warp_incl_scan(sum);
                if (lane == 31) H.wsum[warp] = incl;
                __syncthreads();
                int woff = 0;
                for (int w = 0; w < warp; ++w) woff += H.wsum[w];
                int run = c_below + woff + incl - sum;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int before = run;
                    run += c[u];
                    if (before < k && run >= k) {
                        H.bstar = 4 * tid + u;
                        H.cum_prev = before;
                        H.cum_b = run;
                    }
                }
                if (tid == kHeavyThreads - 1) H.total_in = run;
            }
            __syncthreads();
            const int bstar = H.bstar;
            if (lev == 0) in_radius = H.total_in;
            if (bstar < 0) break;  // fewer than k inside R (level 0), else a numerical edge
            const float v_hi = v_lo + (float)(bstar + 1) * v_w;
            if (H.cum_b <= kCap || lev == 2) {
                Rc = R * radius_of_vol<DIM>(fminf(v_hi, 1.0f)) * 1.00001f;
                break;
            }
            c_below = H.cum_prev;
            v_lo = v_lo + (float)bstar * v_w;
            v_w = v_w / (float)kHeavyBins;
            __syncthreads();
        }

        // ---- outcome: gather + select, or a new radius ------------------------
        float Rnew = -1.0f;
        bool certify = false;
        int reason = 0;
        if (in_radius >= 0 && in_radius < k) {  // too few inside R: grow (bracketed)
            rlo = fmaxf(rlo, R);
            const float g = 1.25f * powf((float)k / (float)max(in_radius, 1), 1.0f / DIM);
            Rnew = R * fminf(fmaxf(g, 1.25f), 4.0f);
            if (rhi > 0.0f && Rnew >= rhi) Rnew = sqrtf(rlo * rhi);
            reason = 1;
        } else {
            if (in_radius > kCap) rhi = (rhi > 0.0f) ? fminf(rhi, R) : R;
            if (Rc < 0.0f) Rc = R;
            const float Rc2 = Rc * Rc;
            if (tid == 0) H.cnt = 0;
            __syncthreads();
            for (int g0 = tid; g0 < total; g0 += 4 * kHeavyThreads) {
                float dd[4];
                uint32_t t[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int g = g0 + u * kHeavyThreads;
                    t[u] = g < total ? slot_of(g) : 0u;
                    dd[u] = g < total ? cand_d2(a, h0, l0, t[u]) : FLT_MAX;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (dd[u] <= Rc2) {
                        const int pos = atomicAdd(&H.cnt, 1);
                        if (pos < kCap) {
                            H.S.d[pos] = dd[u];
                            H.S.i[pos] = (int32_t)t[u];
                        }
                    }
                }
            }
            __syncthreads();
            const int cnt = H.cnt;
#ifdef MG_KNN_DEBUG
            for (int e = tid; e < min(cnt, kCap); e += kHeavyThreads)
                for (int j = 0; j < min(cnt, kCap); ++j)
                    if (j != e && H.S.i[j] == H.S.i[e]) {
                        atomicAdd((unsigned long long *)&a.stats[13], 1ull);
                        atomicMax((unsigned long long *)&a.stats[12], (unsigned long long)qi);
                    }
#endif
            if (cnt < k || cnt > kCap) {
                // rounding at the bin edge or ties finer than the bins: the warp
                // path scans this radius and handles the overflow itself
                Rnew = Rc;
                certify = true;
                reason = 2;
            } else {
                // deterministic buffer order (by slot) before selecting
                int *tmp_i = H.hist;
                float *tmp_d = reinterpret_cast<float *>(H.hist + kCap);
                for (int e = tid; e < cnt; e += kHeavyThreads) {
                    const int32_t me = H.S.i[e];
                    int r = 0;
                    for (int j = 0; j < cnt; ++j) r += H.S.i[j] < me || (H.S.i[j] == me && j < e);
                    tmp_i[r] = me;
                    tmp_d[r] = H.S.d[e];
                }
                __syncthreads();
                for (int e = tid; e < cnt; e += kHeavyThreads) {
                    H.S.i[e] = tmp_i[e];
                    H.S.d[e] = tmp_d[e];
                }
                __syncthreads();
                if (warp == 0) {
                    int32_t *row = a.ngb + (int64_t)qi * k;
                    const float T = select_k<DIM>(H.S, cnt, 1.0f / Rc2, k, row);
                    const float wabs = band_abs(T, query_mag(a.hi, p, a.periodic, a.box_hi));
                    if (T * (1.0f + kBandEps) + 2.0f * wabs > Rc2) {
                        Rnew = sqrtf(T * (1.0f + 2.0f * kBandEps) + 4.0f * wabs) * 1.0001f;
                        certify = true;
                        reason = 3;
                    } else {
                        finish_row(H.S, cnt, T, k, p, qi, a, fr.side, st);
                    }
                }
            }
        }
        if (tid == 0 && Rnew > 0.0f) {
            st.reason[reason - 1] += 1;
            if (a.last_pass) {
                atomicOr(a.qstatus + qi, MG_Q_UNRESOLVED);
                a.radius[qi] = R;
                a.hsml[qi] = -(float)(in_radius + 1000000 * reason);
                st.unres += 1;
            } else {
                a.radius[qi] = certify ? -Rnew : Rnew;
                a.rlo[qi] = rlo;
                a.rhi[qi] = rhi;
                a.qout[atomicAdd(a.qout_count, 1)] = qi;
                st.retry += 1;
            }
        }
        __syncthreads();
    }
    if (tid == 0 && a.stats) {
        if (st.retry) atomicAdd((unsigned long long *)&a.stats[2], (unsigned long long)st.retry);
        if (st.band) atomicAdd((unsigned long long *)&a.stats[3], (unsigned long long)st.band);
        if (st.unres) atomicAdd((unsigned long long *)&a.stats[4], (unsigned long long)st.unres);
        for (int r = 0; r < 3; ++r)
            if (st.reason[r]) atomicAdd((unsigned long long *)&a.stats[6 + r], (unsigned long long)st.reason[r]);
    }
}

template <int DIM, int KPL>
__global__ __launch_bounds__(kHeavyThreads) void k_knn_heavy(const __grid_constant__ KnnArgs a) {
    __shared__ HeavySmem<KPL> H;
    knn_heavy_pass<DIM, KPL>(a, H);
}

// ---- the warp passes as one cooperative launch --------------------------------
// Passes 1 .. npass - 1 of the host loop below in one kernel: each pass runs
// the warp path over the queue the previous pass left, a grid-wide barrier,
// the block-wide path over the heavy queries the warps handed over, and a
// second barrier; the loop ends when a pass starts on an empty queue (every
// block reads the same count after the barrier, so all leave together).  The
// pass's queue pointers are set in a shared copy of the arguments.  Shared
// memory holds the warps' buffers and, in turn, the block-wide path's.
struct PassQueues {
    int32_t *qa, *qb, *counts, *hcounts, *hnext;
    int npass, max_passes;
};

__device__ __forceinline__ void set_pass(KnnArgs &sa, const PassQueues &pq, int pass) {
    sa.qin = pass % 2 ? pq.qa : pq.qb;
    sa.qin_count = pq.counts + (pass - 1);
    sa.qout = pass % 2 ? pq.qb : pq.qa;
    sa.qout_count = pq.counts + pass;
    sa.last_pass = pass == pq.max_passes - 1;
    sa.heavy_count = pq.hcounts + pass;
    sa.heavy_next = pq.hnext + pass;
}

template <int DIM, int KPL>
__global__ __launch_bounds__(kKnnWarps * 32, kKnnMinBlocks) void k_knn_passes(const __grid_constant__ KnnArgs a,
                                                                             const PassQueues pq) {
    static_assert(kKnnWarps * 32 == kHeavyThreads, "one block shape for both paths");
    extern __shared__ __align__(16) unsigned char knn_smem[];
    __shared__ KnnArgs sa;
    cg::grid_group grid = cg::this_grid();
    for (int pass = 1; pass < pq.npass; ++pass) {
        __syncthreads();  // the previous pass is done with sa
        if (threadIdx.x == 0) {
            sa = a;
            set_pass(sa, pq, pass);
        }
        __syncthreads();
        if (__ldcg(sa.qin_count) == 0) break;  // the same value in every block (read at L2)
        if (blockIdx.x == 0 && threadIdx.x == 0 && sa.stats) atomicAdd((unsigned long long *)&sa.stats[0], 1ull);
        knn_warp_pass<DIM, KPL>(sa, knn_smem);
        grid.sync();
        knn_heavy_pass<DIM, KPL>(sa, *reinterpret_cast<HeavySmem<KPL> *>(knn_smem));
        grid.sync();
    }
}

// ---- first pass, one thread per query over a block-shared candidate set --------
// The G queries of a block are consecutive (neighbours in Morton order).  The
// block looks up the cells over the bounding box of its queries' first-radius
// spheres and stages, once, every particle inside the box of some warp's
// spheres into shared memory as its offset from the block centre (FP32, with
// the slot).  Each thread then serves its own query from the staged set:
//   A: offsets compared against R (staged words outside the warp's box are
//      skipped) -> per-thread list of the candidates with d~ <= R;
//   B: 32-bucket histogram of the list in (d~/R)^dim;
//   C: buckets below the k-th neighbour's are taken whole, its bucket is
//      ordered by (d~^2, slot).
// d~ differs from the distance by at most e (a bound from the box size), so the
// set is the exact k nearest when the k-th d~ plus e stays inside R (every
// particle outside the staged boxes is farther than R) and the next d~ is more
// than 2e beyond the k-th (no other particle can change places with it).
// Every other query (too few in radius, a near tie, a crowded boundary
// bucket, a block whose staging overflows, a radius far above the block's
// smallest) goes to the work queue, and the warp passes finish it.  Only the
// rows' slots are written (the order inside a row is the staging order); h is
// solved from them by k_hsml_solve_rows with the warp path's FP32 hi/lo
// distances (cand_d2p).
constexpr int kGroupBins = 32;
constexpr int kGroupList = 96;        // listed candidates per query
constexpr int kGroupBoundary = 8;     // entries of the k-th neighbour's bucket kept per query
constexpr int kGroupUnroll = 4;       // particles per thread per staging round
#ifndef MG_KNN_GROUP_OUTLIER
#define MG_KNN_GROUP_OUTLIER 2.0f
#endif
constexpr float kGroupOutlier = MG_KNN_GROUP_OUTLIER;  // radius above this multiple of the block's smallest: warp path

template <int G, int C>
struct GroupSmem {
    static constexpr int kWarps = G / 32;
    static constexpr int kWords = C / 32;
    static constexpr int kCells = 512;  // local Morton space of an 8 x 8 x 8 cell box
    float sx[C], sy[C], sz[C];          // staged: offsets from the block centre
    uint32_t ss[C];                     // and slots
    float wbox[kWords][6];              // per staged word of 32: min x y z, max x y z
    float qbox[kWarps][6];              // per warp: box of its member queries' spheres
    uint16_t list[kGroupList * G];      // entry e of thread t at list_at(e, t); the
                                        // selected neighbours end up in the first k
    uint16_t bnd[kGroupBoundary * G];   // boundary-bucket staged indices
    float bnd_d[kGroupBoundary * G];    // and their d~^2
    uint8_t hist[kGroupBins * G];       // per-thread bucket counts
    uint32_t cell_a[kCells];            // first slot of each box cell
    uint32_t cell_off[kCells + 1];      // prefix offsets of the cells' particles
    float red[8][kWarps];               // block reductions
    int wtot[2][kWarps];
};

// Entry e of thread t in the per-thread lists (u16): a row of G entries per e,
// the two halves of each 32-bit word held by lanes of different warps, so
// that the 32 lanes of a warp always hit 32 different banks.
__device__ __forceinline__ int list_at(int e, int t) {
    return e * (int)blockDim.x + ((t >> 6) << 6) + ((t & 31) << 1) + ((t >> 5) & 1);
}

// Byte of thread t's counter of bucket b in the per-thread histograms of a
// block of G threads: the four counters b = 4 i .. 4 i + 3 of a thread share
// one 32-bit word, and word i of thread t sits at i * G + t, so that the 32
// lanes of a warp always address 32 different banks whatever their buckets.
template <int G>
__device__ __forceinline__ int hist_at(int b, int t) { return (((b >> 2) * G + t) << 2) + (b & 3); }

// d~^2 between offsets (one expression for every pass; the packed form below
// rounds each half the same way)
template <int DIM>
__device__ __forceinline__ float group_d2(float cx, float cy, float cz, float qx, float qy, float qz) {
    const float dx = __fsub_rn(cx, qx);
    float d2 = __fmul_rn(dx, dx);
    if (DIM > 1) {
        const float dy = __fsub_rn(cy, qy);
        d2 = __fmaf_rn(dy, dy, d2);
    }
    if (DIM > 2) {
        const float dz = __fsub_rn(cz, qz);
        d2 = __fmaf_rn(dz, dz, d2);
    }
    return d2;
}

// Two FP32 lanes in one 64-bit register (element 0 in the low half), with the
// packed arithmetic of sm_100+: each half rounds as the scalar instruction.
__device__ __forceinline__ unsigned long long f2_pack(float v) {
    const unsigned long long b = __float_as_uint(v);
    return b | (b << 32);
}
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b,
                                                     unsigned long long c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// Optional phase cycle counters of the first pass (build with
// -DMG_KNN_GROUP_PROF): stats[10..15] accumulate, over warps, the clock64()
// cycles of set-up and cell lookups, staging, the candidate scan, selection,
// row writes, and hand-over.
#ifdef MG_KNN_GROUP_PROF
#define GROUP_TICK(i) \
    do {              \
        __syncwarp(); \
        gt[i] = clock64(); \
    } while (0)
#else
#define GROUP_TICK(i)
#endif

template <int DIM, int G, int C>
__global__ __launch_bounds__(G) void k_knn_group(KnnArgs a) {
    extern __shared__ __align__(16) unsigned char group_smem[];
    using SM = GroupSmem<G, C>;
    static_assert(G % 64 == 0 && SM::kCells % G == 0, "list_at and the cell split need G = 64 m, G | 512");
    constexpr int NW = SM::kWarps;
    SM &S = *reinterpret_cast<SM *>(group_smem);
    const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
    const int64_t qi = (int64_t)blockIdx.x * G + tid;
    const bool valid = qi < a.nq;
    const Frame fr = load_frame(a.frame);
    const float side = (float)fr.side;
    const float half_side = 0.5f * side;
    const int k = a.k;
#ifdef MG_KNN_GROUP_PROF
    long long gt[7];
#endif
    GROUP_TICK(0);

    int32_t p = 0;
    float4 h0 = make_float4(0.f, 0.f, 0.f, 0.f), l0 = h0;
    float R = 0.0f;
    if (valid) {
        p = a.queries ? a.queries[qi] : (int32_t)qi;
        h0 = a.hi[p];
        l0 = a.lo[p];
        R = a.seed_h[qi] * a.radius_factor;
        if (!(R > 0.0f) || !isfinite(R)) R = side * 1e-3f;
    }
    // ---- members and the block's box (hi parts) --------------------------------
    float v = warp_min(valid ? R : FLT_MAX);
    if (lane == 0) S.red[0][wib] = v;
    __syncthreads();
    float rmin = S.red[0][0];
#pragma unroll
    for (int w = 1; w < NW; ++w) rmin = fminf(rmin, S.red[0][w]);
    const bool mine = valid && R <= kGroupOutlier * rmin;
    float bb[7];
    bb[0] = mine ? h0.x - R : FLT_MAX;
    bb[1] = mine ? h0.y - R : FLT_MAX;
    bb[2] = mine ? h0.z - R : FLT_MAX;
    bb[3] = mine ? -(h0.x + R) : FLT_MAX;
    bb[4] = mine ? -(h0.y + R) : FLT_MAX;
    bb[5] = mine ? -(h0.z + R) : FLT_MAX;
    bb[6] = mine ? -R : FLT_MAX;
#pragma unroll
    for (int i = 0; i < 7; ++i) {
        bb[i] = warp_min(bb[i]);
        if (lane == 0) S.red[1 + i][wib] = bb[i];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 7; ++i) {
        float r = S.red[1 + i][0];
#pragma unroll
        for (int w = 1; w < NW; ++w) r = fminf(r, S.red[1 + i][w]);
        bb[i] = r;
    }
    const float rmax = -bb[6];
    // the hi parts differ from the positions by up to 2^-24 |x|
    float blo[3] = {bb[0], bb[1], bb[2]}, bhi[3] = {-bb[3], -bb[4], -bb[5]};
    float xm = 0.0f;
#pragma unroll
    for (int d = 0; d < DIM; ++d) xm = fmaxf(xm, fmaxf(fabsf(blo[d]), fabsf(bhi[d])));
    const float mg = 1e-5f * rmax + 4e-7f * xm + 1e-30f;
    float ctr[3] = {0.0f, 0.0f, 0.0f}, ext = 0.0f, ehalf = 0.0f;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        blo[d] -= mg;
        bhi[d] += mg;
        ctr[d] = 0.5f * (blo[d] + bhi[d]);
        ext = fmaxf(ext, bhi[d] - blo[d]);
        ehalf = fmaxf(ehalf, fmaxf(fabsf(blo[d] - ctr[d]), fabsf(bhi[d] - ctr[d])));
    }
    // offsets from the centre carry at most ~2^-23 ehalf of rounding per axis,
    // and the hi/lo split of each position ~2^-48 |x| of representation error
    // (2^-46 |x| per axis for a difference, with the low parts' rounding):
    // bound on |d~ - d| for d <= R (twice the analysis)
    const float eg = 1e-6f * ehalf + 3e-7f * rmax + 3e-14f * xm;
    float qx = 0.0f, qy = 0.0f, qz = 0.0f;
    if (DIM > 0) qx = __fadd_rn(__fsub_rn(h0.x, ctr[0]), l0.x);
    if (DIM > 1) qy = __fadd_rn(__fsub_rn(h0.y, ctr[1]), l0.y);
    if (DIM > 2) qz = __fadd_rn(__fsub_rn(h0.z, ctr[2]), l0.z);
    // per-warp box of the member spheres, in offsets
    {
        const float rr = R * (1.0f + 1e-6f) + eg;
        float wb[6];
        wb[0] = mine ? qx - rr : FLT_MAX;
        wb[1] = mine ? qy - rr : FLT_MAX;
        wb[2] = mine ? qz - rr : FLT_MAX;
        wb[3] = mine ? -(qx + rr) : FLT_MAX;
        wb[4] = mine ? -(qy + rr) : FLT_MAX;
        wb[5] = mine ? -(qz + rr) : FLT_MAX;
#pragma unroll
        for (int i = 0; i < 6; ++i) wb[i] = warp_min(wb[i]);
        if (lane == 0) {
#pragma unroll
            for (int i = 0; i < 6; ++i) S.qbox[wib][i] = i < 3 ? wb[i] : -wb[i];
        }
    }

    // ---- box cells: finest level with at most 8 cells per axis over the box ------
    // enumerated in local Morton order, so that consecutive staged particles
    // (a word of 32) are spatially compact and whole words can be skipped
    int L = (int)floorf(log2f(side / ext)) + 3;
    L = max(0, min(kMaxLevel, L));
    int cmin[3], cnum[3];
    for (;;) {
        const float cps = (float)(1u << L), scale = cps / side;
        const float em = 1e-3f + cps * 2.4e-7f;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (d >= DIM) {
                cmin[d] = 0;
                cnum[d] = 1;
                continue;
            }
            const int c0 = max(0, (int)floorf((blo[d] + half_side) * scale - em));
            const int c1 = min((int)cps - 1, (int)floorf((bhi[d] + half_side) * scale + em));
            cmin[d] = c0;
            cnum[d] = max(0, c1 - c0 + 1);
        }
        if ((cnum[0] <= 8 && cnum[1] <= 8 && cnum[2] <= 8) || L == 0) break;
        --L;
    }
    constexpr int ncell = SM::kCells;
    constexpr int CPT = ncell / G;  // cells per thread
    const bool geom_ok = rmin < FLT_MAX && cnum[0] <= 8 && cnum[1] <= 8 && cnum[2] <= 8;
    const float cside = side / (float)(1u << L);
    // cell boxes are compared with the warps' boxes with this slack (FP32 cell
    // corners, key quantisation, offset rounding)
    const float cmarg = 2e-6f * side + 1e-3f * cside;
    __syncthreads();  // the warps' boxes
    GROUP_TICK(1);
    // reason: 0 accepted, 1 too few in radius, 3 k-th too close to R, 4 other
    int reason = 4;
    int cnt = 0;
    float T = 0.0f;
    bool served = false;
    int my_nst = 0;
#ifdef MG_KNN_GROUP_DEBUG
    long long dbg_words = 0, dbg_iter = 0;
#endif
    const float R2 = R * R;
    // Warps still to serve, served gsz at a time from the lowest: a block
    // whose staging overflows is staged again as two halves (re-staging smaller
    // groups costs more than the warp passes take for their queries).
    unsigned todo = (1u << NW) - 1u;
    int gsz = NW;
    while (todo) {
    const unsigned wsel = (((1u << gsz) - 1u) << (__ffs(todo) - 1)) & todo;
    // ---- cells of the box that meet a selected warp's box: ranges, offsets ------
    bool block_ok = geom_ok;
    int tot = 0;
    if (block_ok) {
        uint32_t cnt4[CPT];
        int mine4 = 0;
#pragma unroll
        for (int e = 0; e < CPT; ++e) {
            const int c = CPT * tid + e;
            // local Morton index -> (ix, iy, iz), 3 bits each
            const int ix = (c & 1) | ((c >> 2) & 2) | ((c >> 4) & 4);
            const int iy = ((c >> 1) & 1) | ((c >> 3) & 2) | ((c >> 5) & 4);
            const int iz = ((c >> 2) & 1) | ((c >> 4) & 2) | ((c >> 6) & 4);
            cnt4[e] = 0u;
            S.cell_a[c] = 0u;
            bool use = ix < cnum[0] && iy < cnum[1] && iz < cnum[2];
            if (use) {
                const int ii[3] = {ix, iy, iz};
                float clo[3], chi[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    clo[d] = (float)(cmin[d] + ii[d]) * cside - half_side - ctr[d] - cmarg;
                    chi[d] = clo[d] + cside + 2.0f * cmarg;
                }
                bool any = false;
#pragma unroll
                for (int w = 0; w < NW; ++w) {
                    if (!(wsel >> w & 1u)) continue;
                    bool ov = clo[0] <= S.qbox[w][3] && chi[0] >= S.qbox[w][0];
                    if (DIM > 1) ov = ov && clo[1] <= S.qbox[w][4] && chi[1] >= S.qbox[w][1];
                    if (DIM > 2) ov = ov && clo[2] <= S.qbox[w][5] && chi[2] >= S.qbox[w][2];
                    any = any || ov;
                }
                use = any;
            }
            if (use) {
                uint32_t ca, cb;
                cell_range(a.ci, L, (uint32_t)(cmin[0] + ix), (uint32_t)(cmin[1] + iy), (uint32_t)(cmin[2] + iz), ca,
                           cb);
                S.cell_a[c] = ca;
                cnt4[e] = cb - ca;
            }
            mine4 += (int)cnt4[e];
        }
        const int inc = warp_incl_scan(mine4);
        if (lane == 31) S.wtot[0][wib] = inc;
        __syncthreads();
        int woff = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            const int t = S.wtot[0][w];
            if (w < wib) woff += t;
            tot += t;
        }
        int ex = woff + inc - mine4;
#pragma unroll
        for (int e = 0; e < CPT; ++e) {
            S.cell_off[CPT * tid + e] = (uint32_t)ex;
            ex += (int)cnt4[e];
        }
        if (tid == 0) S.cell_off[ncell] = (uint32_t)tot;
        __syncthreads();
        block_ok = tot <= 32 * C;
    }
    // far more particles than the buffer holds: straight to the halves
    if (geom_ok && 2 * gsz > NW && NW > 1 && tot > 3 * C) {
        gsz >>= 1;
        continue;
    }
    // ---- stage the particles inside some warp's box (deterministic order) -------
    int nst = 0;
    if (block_ok) {
        float qb[NW][6];
#pragma unroll
        for (int w = 0; w < NW; ++w)
#pragma unroll
            for (int i = 0; i < 6; ++i) qb[w][i] = (wsel >> w & 1u) ? S.qbox[w][i] : (i < 3 ? FLT_MAX : -FLT_MAX);
        // rounds of G * kGroupUnroll particles; the slots and loads of the next
        // round are issued before this round's compaction and barrier
        auto fetch = [&](int base, uint32_t(&sl)[kGroupUnroll], float4(&hv)[kGroupUnroll],
                         float4(&lv)[kGroupUnroll]) {
            const int g0 = base + tid * kGroupUnroll;
            int c = 0;
            if (g0 < tot) {
                int hi_c = ncell;
                while (hi_c - c > 1) {
                    const int mid = (c + hi_c) >> 1;
                    if ((int)S.cell_off[mid] <= g0)
                        c = mid;
                    else
                        hi_c = mid;
                }
            }
#pragma unroll
            for (int u = 0; u < kGroupUnroll; ++u) {
                const int g = g0 + u;
                sl[u] = 0xffffffffu;
                if (g < tot) {
                    while ((int)S.cell_off[c + 1] <= g) ++c;
                    sl[u] = S.cell_a[c] + (uint32_t)(g - (int)S.cell_off[c]);
                }
            }
#pragma unroll
            for (int u = 0; u < kGroupUnroll; ++u) {
                if (sl[u] != 0xffffffffu) {
                    hv[u] = a.hi[sl[u]];
                    lv[u] = a.lo[sl[u]];
                } else {
                    hv[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                    lv[u] = hv[u];
                }
            }
        };
        uint32_t slot[kGroupUnroll];
        float4 hb[kGroupUnroll], lb[kGroupUnroll];
        if (tot > 0) fetch(0, slot, hb, lb);
        int round = 0;
        for (int base = 0; base < tot; base += G * kGroupUnroll, ++round) {
            uint32_t slot_n[kGroupUnroll];
            float4 hb_n[kGroupUnroll], lb_n[kGroupUnroll];
            if (base + G * kGroupUnroll < tot) fetch(base + G * kGroupUnroll, slot_n, hb_n, lb_n);
            float ox_[kGroupUnroll], oy_[kGroupUnroll], oz_[kGroupUnroll];
            int nkeep = 0;
            unsigned keepm = 0;
#pragma unroll
            for (int u = 0; u < kGroupUnroll; ++u) {
                float ox = 0.0f, oy = 0.0f, oz = 0.0f;
                if (DIM > 0) ox = __fadd_rn(__fsub_rn(hb[u].x, ctr[0]), lb[u].x);
                if (DIM > 1) oy = __fadd_rn(__fsub_rn(hb[u].y, ctr[1]), lb[u].y);
                if (DIM > 2) oz = __fadd_rn(__fsub_rn(hb[u].z, ctr[2]), lb[u].z);
                ox_[u] = ox;
                oy_[u] = oy;
                oz_[u] = oz;
                bool keep = false;
#pragma unroll
                for (int w = 0; w < NW; ++w) {
                    bool in = ox >= qb[w][0] && ox <= qb[w][3];
                    if (DIM > 1) in = in && oy >= qb[w][1] && oy <= qb[w][4];
                    if (DIM > 2) in = in && oz >= qb[w][2] && oz <= qb[w][5];
                    keep = keep || in;
                }
                keep = keep && slot[u] != 0xffffffffu;
                keepm |= keep ? 1u << u : 0u;
                nkeep += keep ? 1 : 0;
            }
            const int inc = warp_incl_scan(nkeep);
            if (lane == 31) S.wtot[round & 1][wib] = inc;
            __syncthreads();
            int woff = 0, btot = 0;
#pragma unroll
            for (int w = 0; w < NW; ++w) {
                const int t = S.wtot[round & 1][w];
                if (w < wib) woff += t;
                btot += t;
            }
            int pos = nst + woff + inc - nkeep;
#pragma unroll
            for (int u = 0; u < kGroupUnroll; ++u) {
                if (keepm >> u & 1u) {
                    if (pos < C) {
                        S.sx[pos] = ox_[u];
                        S.sy[pos] = oy_[u];
                        S.sz[pos] = oz_[u];
                        S.ss[pos] = slot[u];
                    }
                    ++pos;
                }
            }
            nst += btot;
#pragma unroll
            for (int u = 0; u < kGroupUnroll; ++u) {
                slot[u] = slot_n[u];
                hb[u] = hb_n[u];
                lb[u] = lb_n[u];
            }
        }
    }
    const bool stage_ok = block_ok && nst <= C;
    if (!stage_ok && block_ok && 2 * gsz > NW && NW > 1) {
        gsz >>= 1;
        __syncthreads();
        continue;
    }
    const int nw = (nst + 31) >> 5;
    if (stage_ok) {
        // pad the last word with far-away entries; boxes of the staged words
        for (int j = nst + tid; j < nw * 32; j += G) {
            S.sx[j] = 1e30f;
            S.sy[j] = 1e30f;
            S.sz[j] = 1e30f;
            S.ss[j] = 0u;
        }
        for (int w = tid; w < nw; w += G) {
            float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            const int j1 = min(nst, w * 32 + 32);
            for (int j = w * 32; j < j1; ++j) {
                const float cx = S.sx[j], cy = S.sy[j], cz = S.sz[j];
                mn[0] = fminf(mn[0], cx); mx[0] = fmaxf(mx[0], cx);
                mn[1] = fminf(mn[1], cy); mx[1] = fmaxf(mx[1], cy);
                mn[2] = fminf(mn[2], cz); mx[2] = fmaxf(mx[2], cz);
            }
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                S.wbox[w][i] = mn[i];
                S.wbox[w][3 + i] = mx[i];
            }
        }
    }
    __syncthreads();

    GROUP_TICK(2);
    // ---- per-thread selection ----------------------------------------------------
    const bool act = stage_ok && mine && (wsel >> wib & 1u);
    if (act) {
        served = true;
        my_nst = nst;
    }
    if (stage_ok && (wsel >> wib & 1u)) {
        // A: list the staged candidates with d~ <= R (words outside the warp's box skipped)
        float qb[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) qb[i] = S.qbox[wib][i];
        const float R2a = act ? R2 : -1.0f;
        const unsigned long long QX = f2_pack(qx), QY = f2_pack(qy), QZ = f2_pack(qz), R2A = f2_pack(R2a);
        // a word is scanned when some lane's sphere meets its box (distance
        // from the query to the box against R, with slack for rounding)
        const float R2w = act ? R2 * 1.0001f + 1e-30f : -1.0f;
        KNN_LOOP_HINT
        for (int w = 0; w < nw; ++w) {
            bool ov = S.wbox[w][0] <= qb[3] && S.wbox[w][3] >= qb[0];
            if (DIM > 1) ov = ov && S.wbox[w][1] <= qb[4] && S.wbox[w][4] >= qb[1];
            if (DIM > 2) ov = ov && S.wbox[w][2] <= qb[5] && S.wbox[w][5] >= qb[2];
            if (!ov) continue;
            {
                const float ex = fmaxf(0.0f, fmaxf(S.wbox[w][0] - qx, qx - S.wbox[w][3]));
                float bd2 = ex * ex;
                if (DIM > 1) {
                    const float ey = fmaxf(0.0f, fmaxf(S.wbox[w][1] - qy, qy - S.wbox[w][4]));
                    bd2 = fmaf(ey, ey, bd2);
                }
                if (DIM > 2) {
                    const float ez = fmaxf(0.0f, fmaxf(S.wbox[w][2] - qz, qz - S.wbox[w][5]));
                    bd2 = fmaf(ez, ez, bd2);
                }
                if (!__any_sync(0xffffffffu, bd2 <= R2w)) continue;
            }
#ifdef MG_KNN_GROUP_DEBUG
            ++dbg_words;
#endif
            // the word's 32 distances first (independent loads, two per packed
            // instruction), then the list; bit b set when R^2 - d~^2 >= 0
            uint32_t mp[4] = {0u, 0u, 0u, 0u};
            const ulonglong2 *X = reinterpret_cast<const ulonglong2 *>(S.sx + w * 32);
            const ulonglong2 *Y = reinterpret_cast<const ulonglong2 *>(S.sy + w * 32);
            const ulonglong2 *Z = reinterpret_cast<const ulonglong2 *>(S.sz + w * 32);
#pragma unroll
            for (int b4 = 0; b4 < 8; ++b4) {
                const ulonglong2 xv = X[b4];
                ulonglong2 yv, zv;
                if (DIM > 1) yv = Y[b4];
                if (DIM > 2) zv = Z[b4];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const unsigned long long dx = f2_sub(h ? xv.y : xv.x, QX);
                    unsigned long long d2 = f2_mul(dx, dx);
                    if (DIM > 1) {
                        const unsigned long long dy = f2_sub(h ? yv.y : yv.x, QY);
                        d2 = f2_fma(dy, dy, d2);
                    }
                    if (DIM > 2) {
                        const unsigned long long dz = f2_sub(h ? zv.y : zv.x, QZ);
                        d2 = f2_fma(dz, dz, d2);
                    }
                    const unsigned long long df = f2_sub(R2A, d2);
                    const int b = 4 * b4 + 2 * h;
                    mp[(2 * h) & 3] |= ((~(uint32_t)df) >> 31) << b;
                    mp[(2 * h + 1) & 3] |= ((~(uint32_t)(df >> 32)) >> 31) << (b + 1);
                }
            }
            uint32_t m = (mp[0] | mp[1]) | (mp[2] | mp[3]);
#ifdef MG_KNN_GROUP_DEBUG
            dbg_iter += __reduce_max_sync(0xffffffffu, (unsigned)__popc(m));
#endif
            while (m) {
                const int b = __ffs(m) - 1;
                m &= m - 1;
                if (cnt < kGroupList) S.list[list_at(cnt, tid)] = (uint16_t)(w * 32 + b);
                ++cnt;
            }
        }
    }
    GROUP_TICK(3);
    if (act) {
        if (cnt < k) {
            reason = 1;
        } else if (cnt < kGroupList) {
            // B: histogram of the list in 32 buckets of d~^2 / R^2
            const float bscale = 32.0f / R2;
#pragma unroll
            for (int b = 0; b < kGroupBins; ++b) S.hist[hist_at<G>(b, tid)] = 0;
            KNN_LOOP_HINT
            for (int e0 = 0; e0 < cnt; e0 += 4) {
                int bk[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int e = min(e0 + u, cnt - 1);
                    const int j = S.list[list_at(e, tid)];
                    const float d2 = group_d2<DIM>(S.sx[j], S.sy[j], S.sz[j], qx, qy, qz);
                    bk[u] = e0 + u < cnt ? min(kGroupBins - 1, (int)(d2 * bscale)) : -1;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (bk[u] >= 0) ++S.hist[hist_at<G>(bk[u], tid)];
            }
            int cum = 0, bstar = kGroupBins - 1, c_lo = 0, m_b = 0;
            KNN_LOOP_HINT
            for (int b = 0; b < kGroupBins; ++b) {
                const int h = S.hist[hist_at<G>(b, tid)];
                if (cum + h >= k) {
                    bstar = b;
                    c_lo = cum;
                    m_b = h;
                    break;
                }
                cum += h;
            }
            if (m_b <= kGroupBoundary) {
                // C: buckets below taken whole, the boundary bucket kept aside
                int nsure = 0, nb = 0;
                float nextmin = R2;  // anything not listed lies beyond R
                KNN_LOOP_HINT
                for (int e0 = 0; e0 < cnt; e0 += 4) {
                    int jj[4], bk[4];
                    float dd[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int e = min(e0 + u, cnt - 1);
                        jj[u] = S.list[list_at(e, tid)];
                        dd[u] = group_d2<DIM>(S.sx[jj[u]], S.sy[jj[u]], S.sz[jj[u]], qx, qy, qz);
                        bk[u] = e0 + u < cnt ? min(kGroupBins - 1, (int)(dd[u] * bscale)) : kGroupBins;
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        if (bk[u] < bstar) {
                            if (nsure < c_lo) S.list[list_at(nsure, tid)] = (uint16_t)jj[u];
                            ++nsure;
                        } else if (bk[u] == bstar) {
                            if (nb < m_b) {
                                S.bnd[nb * G + tid] = (uint16_t)jj[u];
                                S.bnd_d[nb * G + tid] = dd[u];
                            }
                            ++nb;
                        } else if (bk[u] < kGroupBins) {
                            nextmin = fminf(nextmin, dd[u]);
                        }
                    }
                }
                // the r smallest of the boundary bucket by (d~^2, slot), then the
                // next one; the counts of this pass must repeat the histogram's
                const int r = nsure == c_lo && nb == m_b ? k - c_lo : 0;
                uint32_t taken = 0;
                float nxt = nextmin;
                if (r > 0) {
                    KNN_LOOP_HINT
                    for (int i = 0; i <= r && i < nb; ++i) {
                        float best = FLT_MAX;
                        uint32_t bslot = 0xffffffffu;
                        int bi = 0;
                        KNN_LOOP_HINT
                        for (int e = 0; e < nb; ++e) {
                            if (taken >> e & 1u) continue;
                            const float dv = S.bnd_d[e * G + tid];
                            const uint32_t sl = S.ss[S.bnd[e * G + tid]];
                            if (dv < best || (dv == best && sl < bslot)) {
                                best = dv;
                                bslot = sl;
                                bi = e;
                            }
                        }
                        if (i < r) {
                            taken |= 1u << bi;
                            S.list[list_at(c_lo + i, tid)] = S.bnd[bi * G + tid];
                            T = best;
                        } else {
                            nxt = fminf(nxt, best);
                        }
                    }
                    // exact set: the k-th stays inside R by more than the error
                    // bound, and the next candidate is more than twice the bound
                    // beyond the k-th
                    const float e2 = 1.01f * eg + 2e-7f * R;
                    const float dT = sqrtf(T), dN = sqrtf(nxt);
                    if (dT + 2.0f * e2 > R)
                        reason = 3;
                    else if (dN - dT > 2.0f * e2)
                        reason = 0;
                }
            }
        }
    }

    GROUP_TICK(4);
    // ---- rows of the accepted queries (coalesced, one row per warp step) ---------
    const unsigned acc = __ballot_sync(0xffffffffu, act && reason == 0);
    if (acc) {
        // the rows' slots only: h is solved from them afterwards
#pragma unroll 4
        for (int rr = 0; rr < 32; ++rr) {
            if (!(acc >> rr & 1u)) continue;
            const int64_t q = (int64_t)blockIdx.x * G + wib * 32 + rr;
            if (lane < k) {
                const int j = S.list[list_at(lane, wib * 32 + rr)];
                const uint32_t t = S.ss[j];
                a.ngb[q * k + lane] = (int32_t)t;
            }
        }
    }
    todo &= ~wsel;
    __syncthreads();  // the next group restages the shared buffers
    }
    GROUP_TICK(5);
    // ---- everything else goes to the warp passes -----------------------------------
    const bool push = valid && !(served && reason == 0);
    if (push) {
        float Rnew = R;
        if (served && reason == 1) {
            const float g = 1.25f * powf((float)k / (float)max(cnt, 1), 1.0f / DIM);
            Rnew = R * fminf(fmaxf(g, 1.25f), 4.0f);
        } else if (served && reason == 3) {
            Rnew = fmaxf(R, sqrtf(T) + 4.0f * (1.01f * eg + 2e-7f * R)) * 1.0001f;
        }
        a.radius[qi] = Rnew;
        a.rlo[qi] = 0.0f;
        a.rhi[qi] = 0.0f;
    }
    const unsigned pm = __ballot_sync(0xffffffffu, push);
    if (pm) {
        int base = 0;
        if (lane == 0) base = atomicAdd(a.qout_count, __popc(pm));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (push) a.qout[base + __popc(pm & ((1u << lane) - 1u))] = (int32_t)qi;
    }
#ifdef MG_KNN_GROUP_PROF
    GROUP_TICK(6);
    if (lane == 0 && a.stats)
        for (int i = 0; i < 6; ++i) atomicAdd((unsigned long long *)&a.stats[10 + i], (unsigned long long)(gt[i + 1] - gt[i]));
#endif
#ifdef MG_KNN_GROUP_DEBUG
    // [10] blocks whose staging failed, [11] words scanned summed over warps,
    // [12] member queries pushed for another reason, [13] outliers, [14]
    // listed candidates summed over members, [15] list-append iterations
    // summed over warps
    if (a.stats) {
        const int r4 = __popc(__ballot_sync(0xffffffffu, served && reason == 4));
        const int ol = __popc(__ballot_sync(0xffffffffu, valid && !mine));
        const int64_t lc = warp_sum<int64_t>(served ? (int64_t)cnt : 0);
        if (tid == 0 && !geom_ok) atomicAdd((unsigned long long *)&a.stats[10], 1ull);
        if (lane == 0) {
            atomicAdd((unsigned long long *)&a.stats[11], (unsigned long long)dbg_words);
            atomicAdd((unsigned long long *)&a.stats[15], (unsigned long long)dbg_iter);
        }
        if (lane == 0) {
            if (r4) atomicAdd((unsigned long long *)&a.stats[12], (unsigned long long)r4);
            if (ol) atomicAdd((unsigned long long *)&a.stats[13], (unsigned long long)ol);
            if (lc) atomicAdd((unsigned long long *)&a.stats[14], (unsigned long long)lc);
        }
    }
#endif
    // statistics: staged candidates per member query, retries and their reasons
    if (a.stats) {
        const int64_t cand = warp_sum<int64_t>(served ? (int64_t)my_nst : 0);
        const int n1 = __popc(__ballot_sync(0xffffffffu, push && served && reason == 1));
        const int n3 = __popc(__ballot_sync(0xffffffffu, push && served && reason == 3));
        if (lane == 0) {
            if (cand) atomicAdd((unsigned long long *)&a.stats[1], (unsigned long long)cand);
            if (pm) atomicAdd((unsigned long long *)&a.stats[2], (unsigned long long)__popc(pm));
            if (n1) atomicAdd((unsigned long long *)&a.stats[6], (unsigned long long)n1);
            if (n3) atomicAdd((unsigned long long *)&a.stats[8], (unsigned long long)n3);
        }
    }
}

// ---- smoothing length: one thread per query ------------------------------------
// hsml_newton (mg_hsml.cuh) solves each query's row.

// Newton iterations, summed per warp into stats[5]
__device__ __forceinline__ void add_newton_steps(int it, int64_t *stats) {
    int wsum = it;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
    if ((threadIdx.x & 31) == 0 && wsum && stats) atomicAdd((unsigned long long *)&stats[5], (unsigned long long)wsum);
}

// From given squared distances (nq rows of k).  KR > 0: the k <= KR distances
// are loaded once (16-byte loads when k is a multiple of 4) and kept in
// registers for all Newton steps; KR == 0: any k, read again on each step.
template <int DIM, int KR>
__global__ __launch_bounds__(128) void k_hsml_solve(const float *__restrict__ dsel, const int32_t *__restrict__ qstatus,
                                                    int64_t nq, int k, float *__restrict__ hsml,
                                                    float *__restrict__ hsml_lo, int64_t *__restrict__ stats) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int it = 0;
    if (q < nq && !(qstatus && (qstatus[q] & MG_Q_UNRESOLVED))) {
        const float *row = dsel + q * k;
        constexpr int KN = KR > 0 ? KR : 1;
        float dr[KN];
        if (KR > 0) {
            if ((k & 3) == 0) {
#pragma unroll
                for (int j = 0; j < KN; j += 4) {
                    if (j < k) {
                        const float4 v = __ldg(reinterpret_cast<const float4 *>(row + j));
                        dr[j] = sqrtf(v.x);
                        dr[j + 1] = sqrtf(v.y);
                        dr[j + 2] = sqrtf(v.z);
                        dr[j + 3] = sqrtf(v.w);
                    }
                }
            } else {
#pragma unroll
                for (int j = 0; j < KN; ++j)
                    if (j < k) dr[j] = sqrtf(__ldg(row + j));
            }
        }
        float hl = 0.0f;
        hsml[q] = hsml_newton<DIM, KR>([&](int j) -> float { return KR > 0 ? dr[j] : sqrtf(row[j]); }, k, it, &hl);
        if (hsml_lo) hsml_lo[q] = hl;
        it += 1;
    }
    add_newton_steps(it, stats);
}

// Float-float distance between a query and a neighbour from their hi/lo
// positions (hb, lb already loaded): separations by TwoSum (sep1_ff /
// wrap1_ff), squared and summed in float-float, one Newton correction of the
// square root.
template <int DIM>
__device__ __forceinline__ ff dist_ff(const float4 &h0, const float4 &l0, const float4 &hb, const float4 &lb,
                                      bool periodic, float box_hi, float box_lo) {
    const float bh[3] = {hb.x, hb.y, hb.z}, bl[3] = {lb.x, lb.y, lb.z};
    const float ah[3] = {h0.x, h0.y, h0.z}, al[3] = {l0.x, l0.y, l0.z};
    ff r2 = ff{0.0f, 0.0f};
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
        float l;
        const float d = periodic ? wrap1_ff(bh[c], ah[c], bl[c], al[c], box_hi, box_lo, l)
                                 : sep1_ff(bh[c], ah[c], bl[c], al[c], l);
        r2 = ff_add(r2, ff_sqr(ff{d, l}));
    }
    return ff_sqrt(r2);
}

// h from the neighbour rows (k <= 32), the search writing only the rows: the
// row's distances in FP32 (cand_d2p, the search's own expression) kept in
// registers, the Newton solve unrolled over them.
template <int DIM>
__global__ __launch_bounds__(128) void k_hsml_solve_rows(const int32_t *__restrict__ ngb,
                                                         const int32_t *__restrict__ queries,
                                                         const float4 *__restrict__ hi, const float4 *__restrict__ lo,
                                                         bool periodic, float box_hi, float box_lo,
                                                         const int32_t *__restrict__ qstatus, int64_t nq, int k,
                                                         float *__restrict__ hsml, int64_t *__restrict__ stats) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int it = 0;
    if (q < nq && !(qstatus && (qstatus[q] & MG_Q_UNRESOLVED))) {
        const int32_t p = queries ? queries[q] : (int32_t)q;
        const float4 h0 = hi[p], l0 = lo[p];
        const int32_t *row = ngb + q * k;
        int32_t t[32];
        if ((k & 3) == 0) {
#pragma unroll
            for (int j = 0; j < 32; j += 4) {
                if (j < k) {
                    const int4 v = __ldg(reinterpret_cast<const int4 *>(row + j));
                    t[j] = v.x;
                    t[j + 1] = v.y;
                    t[j + 2] = v.z;
                    t[j + 3] = v.w;
                }
            }
        } else {
#pragma unroll
            for (int j = 0; j < 32; ++j)
                if (j < k) t[j] = __ldg(row + j);
        }
        float dr[32];
#pragma unroll
        for (int j = 0; j < 32; ++j)
            if (j < k) dr[j] = sqrtf(cand_d2p(hi, lo, periodic, box_hi, box_lo, h0, l0, (uint32_t)t[j]));
        hsml[q] = hsml_newton<DIM, 32>([&](int j) -> float { return dr[j]; }, k, it);
        it += 1;
    }
    add_newton_steps(it, stats);
}

// Float-float h: the row's distances are computed in float-float as they are
// gathered (one gather), the FP32 Newton solve runs on their high parts, and
// one Newton step with the neighbour count in float-float (hsml_polish_ff)
// gives h = hsml + hsml_lo to ~1e-12.  An FP32-only h (~1e-7: FP32 distances
// and kernel values limit it on rows where a few neighbours dominate the
// slope) moved some order-1 derivatives by 1.6e-5.  The distances wait in
// shared memory (this thread's column) and every loop over them stays
// rolled: unrolled over 32 register-resident float-float distances, the
// kernel outgrew the instruction cache and stalled on instruction fetch.
// The hi/lo positions carry ~2^-48 |x| of representation error, ~1.2e-14 |x|
// of a distance: a row whose largest distance is below ~1e-4 of |x| (|x| the
// query's frame-relative coordinates, or the box side) would lose h beyond
// 1e-10 to it, so its distances are recomputed from the FP64 positions
// (d2_exact, the parity metric) before the solve.
template <int DIM>
__global__ __launch_bounds__(128) void k_hsml_solve_rows_ff(const int32_t *__restrict__ ngb,
                                                            const int32_t *__restrict__ queries,
                                                            const float4 *__restrict__ hi,
                                                            const float4 *__restrict__ lo, bool periodic, float box_hi,
                                                            float box_lo, const double *__restrict__ pos64,
                                                            double box64, const int32_t *__restrict__ qstatus,
                                                            int64_t nq, int k, float *__restrict__ hsml,
                                                            float *__restrict__ hsml_lo, int64_t *__restrict__ stats) {
    __shared__ float sdh[32 * 128], sdl[32 * 128];  // [neighbour][thread]
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int it = 0;
    if (q < nq && !(qstatus && (qstatus[q] & MG_Q_UNRESOLVED))) {
        const int32_t p = queries ? queries[q] : (int32_t)q;
        const float4 h0 = hi[p], l0 = lo[p];
        const int32_t *row = ngb + q * k;
        const int tx = threadIdx.x;
        float dmax = 0.0f;
        if ((k & 3) == 0) {
#pragma unroll 2
            for (int j = 0; j < k; j += 4) {
                const int4 v = __ldg(reinterpret_cast<const int4 *>(row + j));
                const int32_t tv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const ff d = dist_ff<DIM>(h0, l0, hi[tv[u]], lo[tv[u]], periodic, box_hi, box_lo);
                    sdh[(j + u) * 128 + tx] = d.hi;
                    sdl[(j + u) * 128 + tx] = d.lo;
                    dmax = fmaxf(dmax, d.hi);
                }
            }
        } else {
#pragma unroll 4
            for (int j = 0; j < k; ++j) {
                const int32_t s = __ldg(row + j);
                const ff d = dist_ff<DIM>(h0, l0, hi[s], lo[s], periodic, box_hi, box_lo);
                sdh[j * 128 + tx] = d.hi;
                sdl[j * 128 + tx] = d.lo;
                dmax = fmaxf(dmax, d.hi);
            }
        }
        float xq = fmaxf(fabsf(h0.x), fmaxf(fabsf(h0.y), fabsf(h0.z)));
        if (periodic) xq = fmaxf(xq, box_hi);
        if (1.2e-14f * xq > 1e-10f * dmax) {
#pragma unroll 1
            for (int j = 0; j < k; ++j) {
                const double d2 = d2_exact(pos64, p, __ldg(row + j), periodic, box64);
                const float d2h = (float)d2;
                const ff d = ff_sqrt(ff{d2h, (float)(d2 - (double)d2h)});
                sdh[j * 128 + tx] = d.hi;
                sdl[j * 128 + tx] = d.lo;
            }
        }
        const float h32 = hsml_newton<DIM, 0, true>([&](int j) -> float { return sdh[j * 128 + tx]; }, k, it);
        it += 1;
        const ff h = hsml_polish_ff<DIM, 1, 0>([&](int j) { return ff{sdh[j * 128 + tx], sdl[j * 128 + tx]}; }, k,
                                               h32);
        hsml[q] = h.hi;
        hsml_lo[q] = h.lo;
    }
    add_newton_steps(it, stats);
}

// Squared distances of the neighbour rows (k > 32, for k_hsml_solve<DIM, 0>).
__global__ __launch_bounds__(256) void k_row_d2(const int32_t *__restrict__ ngb, const int32_t *__restrict__ queries,
                                                const float4 *__restrict__ hi, const float4 *__restrict__ lo,
                                                bool periodic, float box_hi, float box_lo, int64_t nq, int k,
                                                float *__restrict__ d2) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= nq * (int64_t)k) return;
    const int64_t q = e / k;
    const int32_t p = queries ? queries[q] : (int32_t)q;
    d2[e] = cand_d2p(hi, lo, periodic, box_hi, box_lo, hi[p], lo[p], (uint32_t)ngb[e]);
}

template <int DIM>
static void launch_hsml_solve(unsigned hb, cudaStream_t st, const float *dsel, const int32_t *qstatus, int64_t nq,
                              int k, float *hsml, int64_t *stats) {
    if (k <= 32)
        k_hsml_solve<DIM, 32><<<hb, 128, 0, st>>>(dsel, qstatus, nq, k, hsml, nullptr, stats);
    else
        k_hsml_solve<DIM, 0><<<hb, 128, 0, st>>>(dsel, qstatus, nq, k, hsml, nullptr, stats);
}

// h of every resolved query from its neighbour row; dsel: nq * k scratch for k > 32
// hsml_lo (may be NULL): the low part of each h (float-float: k <= 32 from
// float-float distances; k > 32 the Newton solve's last step kept as an
// unevaluated sum, ~1e-8)
template <int DIM>
static int launch_hsml_rows(cudaStream_t st, const KnnArgs &a, const int32_t *qstatus, int64_t nq, int k,
                            float *dsel, float *hsml, float *hsml_lo, int64_t *stats) {
    const unsigned hb = (unsigned)((nq + 127) / 128);
    if (k <= 32) {
        if (hsml_lo)
            k_hsml_solve_rows_ff<DIM><<<hb, 128, 0, st>>>(a.ngb, a.queries, a.hi, a.lo, a.periodic, a.box_hi,
                                                          a.box_lo, a.pos64, a.box64, qstatus, nq, k, hsml, hsml_lo,
                                                          stats);
        else
            k_hsml_solve_rows<DIM><<<hb, 128, 0, st>>>(a.ngb, a.queries, a.hi, a.lo, a.periodic, a.box_hi, a.box_lo,
                                                       qstatus, nq, k, hsml, stats);
        MG_CHECK_LAUNCH();
        return MG_OK;
    }
    const int64_t ne = nq * (int64_t)k;
    k_row_d2<<<(unsigned)((ne + 255) / 256), 256, 0, st>>>(a.ngb, a.queries, a.hi, a.lo, a.periodic, a.box_hi,
                                                            a.box_lo, nq, k, dsel);
    MG_CHECK_LAUNCH();
    k_hsml_solve<DIM, 0><<<hb, 128, 0, st>>>(dsel, qstatus, nq, k, hsml, hsml_lo, stats);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

__global__ void k_count_pass(const int32_t *qcount, int64_t *stats) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && *qcount > 0) atomicAdd((unsigned long long *)&stats[0], 1ull);
}

// ---- plain seed --------------------------------------------------------------
// h from the particle count of the query's adaptive cell: the finest level whose
// cell around the query still holds at least max(2, k/4) particles.
__device__ __forceinline__ void own_cell_range(const CellIndex &ci, uint64_t key, int L, uint32_t &a, uint32_t &b) {
    cell_lookup(ci, L, key >> (3 * (kKeyBits - L)), a, b);
}

// Finest level at which the Morton keys a and b share a cell (kMaxLevel at most).
__device__ __forceinline__ int common_level(uint64_t a, uint64_t b) {
    const uint64_t x = a ^ b;
    if (x == 0) return kMaxLevel;
    const int hb = 63 - __clzll((long long)x);  // highest differing bit; level l uses bits >= 3 (21 - l)
    return min(kMaxLevel, (62 - hb) / 3);
}

// Adaptive level of slot p without cell lookups: the own cell at level l holds
// >= cmin particles exactly when some run of cmin consecutive slots containing
// p shares its level-l prefix, i.e. when the first and last keys of that run do
// (the keys are sorted).  Window w (0 <= w < cmin) is the run starting at
// p - w; the level is the largest common level over the windows.
__device__ __forceinline__ int window_level(const uint64_t *__restrict__ keys, int64_t n, int64_t p, int cmin, int w) {
    const int64_t s = p - w;
    if (w >= cmin || s < 0 || s + cmin - 1 >= n) return 0;
    return common_level(keys[s], keys[s + cmin - 1]);
}

__global__ void k_seed_plain(const CellIndex ci, int64_t n, const double *__restrict__ framep, const int32_t *queries,
                             int64_t nq, int k, int dim, float *__restrict__ seed_h) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int32_t p = queries ? queries[q] : (int32_t)q;
    const int cmin = max(2, k / 4);
    int L = 0;
    for (int w = 0; w < cmin; ++w) L = max(L, window_level(ci.keys, n, p, cmin, w));
    uint32_t a0, b0;
    own_cell_range(ci, ci.keys[p], L, a0, b0);
    const uint32_t cnt = b0 - a0;
    // side / 2^L: the power-of-two scaling is exact, so scaling the FP32
    // rounding of side equals rounding the FP64 quotient (no FP64 division,
    // whose rate on this GPU made it the seed passes' bottleneck)
    const float s = ldexpf((float)framep[3], -L);
    const float c = (float)max(cnt, 1u);
    float h;
    if (dim == 3)
        h = s * cbrtf(3.0f * k / (4.0f * 3.14159265f * c));
    else if (dim == 2)
        h = s * sqrtf(k / (3.14159265f * c));
    else
        h = s * k / (2.0f * c);
    seed_h[q] = h;
}

// ---- seed-network features -----------------------------------------------------
// One warp per run of consecutive queries.  The adaptive level (finest level
// whose cell around the query holds >= max(2, k/4) particles) comes from the
// keys of the neighbouring slots (window_level), one window per lane.  Features: log2(1 + count) of
// the 27 cells around the query at levels L+1 and L (finer first); a query in
// the same level-(L+1) cell as the previous one reuses its values.
__global__ __launch_bounds__(256) void k_seed_features(const CellIndex ci, int64_t n,
                                                       const double *__restrict__ framep,
                                                       const int32_t *queries, int64_t nq, int k,
                                                       int dim, int periodic,
                                                       uint16_t *__restrict__ feat,
                                                       float *__restrict__ cell_side) {
    const int lane = threadIdx.x & 31;
    const int64_t gwarp = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t per = (nq + nwarps - 1) / nwarps;
    const int64_t q0 = gwarp * per, q1 = min(nq, q0 + per);
    const int cmin = max(2, k / 4);
    const float side = (float)framep[3];
    int cachedL = -1;
    uint64_t cachedCell = ~0ull;
    uint32_t w0 = 0, w1 = 0;  // packed bf16 pairs of this lane's two output columns
    for (int64_t q = q0; q < q1; ++q) {
        const int32_t p = queries ? queries[q] : (int32_t)q;
        const uint64_t key = ci.keys[p];
        // adaptive level from runs of cmin consecutive keys (lane w: the run
        // starting at p - w)
        int L = 0;
        for (int w = lane; w < cmin; w += 32) L = max(L, window_level(ci.keys, n, p, cmin, w));
        L = (int)__reduce_max_sync(0xffffffffu, (unsigned)L);
        const int Lf = min(L + 1, kMaxLevel);
        const uint64_t cellF = key >> (3 * (kKeyBits - Lf));
        if (L != cachedL || cellF != cachedCell) {
            cachedL = L;
            cachedCell = cellF;
            uint32_t c21[3] = {0, 0, 0};
            for (int b = 0; b < kKeyBits; ++b) {
                c21[0] |= (uint32_t)((key >> (3 * b)) & 1ull) << b;
                c21[1] |= (uint32_t)((key >> (3 * b + 1)) & 1ull) << b;
                c21[2] |= (uint32_t)((key >> (3 * b + 2)) & 1ull) << b;
            }
            float vals[2] = {0.0f, 0.0f};
            for (int lev = 0; lev < 2; ++lev) {
                const int LL = lev == 0 ? Lf : L;
                const int M = 1 << LL;
                if (lane < 27) {
                    const int off[3] = {lane % 3 - 1, (lane / 3) % 3 - 1, lane / 9 - 1};
                    int g[3];
                    bool inside = true;
                    for (int d = 0; d < 3; ++d) {
                        g[d] = (int)(c21[d] >> (kKeyBits - LL)) + (d < dim ? off[d] : 0);
                        if (d >= dim && off[d] != 0) inside = false;  // collapsed axis
                        if (periodic)
                            g[d] = ((g[d] % M) + M) % M;
                        else if (g[d] < 0 || g[d] >= M)
                            inside = false;
                    }
                    if (inside) {
                        uint32_t ca, cb;
                        cell_range(ci, LL, (uint32_t)g[0], (uint32_t)g[1], (uint32_t)g[2], ca, cb);
                        // the fast intrinsic: the feature is rounded to BF16
                        // (8 bits) for the network, far coarser than its error
                        vals[lev] = __log2f(1.0f + (float)(cb - ca));
                    }
                }
            }
            // columns: [0, 27) level L+1, [27, 54) level L, [54, 64) zero
            float c0 = 0.0f, c1 = 0.0f;
            {
                const int idx0 = lane, idx1 = lane + 32;
                const float x0 = __shfl_sync(0xffffffffu, vals[0], idx0 < 27 ? idx0 : 0);
                const float y0 = __shfl_sync(0xffffffffu, vals[1], (idx0 >= 27 && idx0 < 54) ? idx0 - 27 : 0);
                const float y1 = __shfl_sync(0xffffffffu, vals[1], (idx1 < 54) ? idx1 - 27 : 0);
                c0 = idx0 < 27 ? x0 : y0;
                c1 = idx1 < 54 ? y1 : 0.0f;
            }
            auto bf = [](float v) -> uint32_t {
                uint32_t bits = __float_as_uint(v);
                bits += 0x7fffu + ((bits >> 16) & 1u);
                return bits >> 16;
            };
            w0 = bf(c0);
            w1 = bf(c1);
        }
        uint16_t *row = feat + q * MG_MLP_IN_PAD;
        row[lane] = (uint16_t)w0;
        row[lane + 32] = (uint16_t)w1;
        if (lane == 0) cell_side[q] = ldexpf(side, -L);  // = (float)(side / 2^L), exact scaling
    }
}

// ---- smoothing lengths, densities and volumes in row order ----------------------
// src/meshoid/Meshoid.py:169-170: density = des_ngb m / (volnorm h^dim),
// vol = m / density, volnorm = 2, pi, 4 pi / 3 in 1/2/3-D.
__global__ void k_density(const int32_t *__restrict__ out_rows, const float *__restrict__ hsml,
                          const float *__restrict__ hsml_lo, int64_t nq,
                          const double *__restrict__ m_rows, double des_ngb, double inv_ngb, int dim,
                          double volnorm, double *__restrict__ h_out, double *__restrict__ density,
                          double *__restrict__ vol) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int64_t r = out_rows ? (int64_t)out_rows[q] : q;
    const double h = (double)hsml[q] + (hsml_lo ? (double)hsml_lo[q] : 0.0);
    const double hd = dim == 3 ? h * h * h : (dim == 2 ? h * h : h);
    const double m = m_rows ? m_rows[r] : 1.0;
    const double v = volnorm * hd;  // vol = m / density = volnorm h^dim / des_ngb
    h_out[r] = h;
    // one FP64 division per particle (they run at a small fraction of the
    // FP32 rate on this GPU); the volume takes 1 / des_ngb (from the host) as
    // a product
    if (density) density[r] = des_ngb * m / v;
    if (vol) vol[r] = v * inv_ngb;
}

// ---- per-row FP64 distances, sorted ---------------------------------------------
__global__ __launch_bounds__(256) void k_neighbor_dist(const double *__restrict__ pos64,
                                                       const int32_t *__restrict__ order,
                                                       const int32_t *queries, int64_t nq,
                                                       const int32_t *__restrict__ ngb, int k,
                                                       bool periodic, double box,
                                                       int64_t *__restrict__ out_idx,
                                                       double *__restrict__ out_d) {
    const int lane = threadIdx.x & 31;
    const int64_t q = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= nq) return;
    const int32_t p = queries ? queries[q] : (int32_t)q;
    const int32_t *row = ngb + q * k;
    // k <= 128: up to 4 per lane; sort each 32-chunk, then merge by selection
    double key[MG_MAX_K / 32];
    int32_t tie[MG_MAX_K / 32];
    const int kpl = (k + 31) >> 5;
#pragma unroll
    for (int j = 0; j < MG_MAX_K / 32; ++j) {
        const int e = lane + 32 * j;
        if (j < kpl && e < k) {
            const int32_t s = row[e];
            key[j] = d2_exact(pos64, p, s, periodic, box);
            tie[j] = order[s];
        } else {
            key[j] = DBL_MAX;
            tie[j] = INT_MAX;
        }
    }
    // k-way selection: repeatedly extract the minimum (k <= 128)
    for (int o = 0; o < k; ++o) {
        double bk = DBL_MAX;
        int32_t bt = INT_MAX;
        int bj = -1;
#pragma unroll
        for (int j = 0; j < MG_MAX_K / 32; ++j)
            if (key[j] < bk || (key[j] == bk && tie[j] < bt)) {
                bk = key[j];
                bt = tie[j];
                bj = j;
            }
        double wk = bk;
        int32_t wt = bt;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            double ok = __shfl_xor_sync(0xffffffffu, wk, off);
            int32_t ot = __shfl_xor_sync(0xffffffffu, wt, off);
            if (ok < wk || (ok == wk && ot < wt)) {
                wk = ok;
                wt = ot;
            }
        }
        if (bj >= 0 && bk == wk && bt == wt) {
#pragma unroll
            for (int j = 0; j < MG_MAX_K / 32; ++j)
                if (j == bj) {
                    key[j] = DBL_MAX;
                    tie[j] = INT_MAX;
                }
        }
        if (lane == 0) {
            out_idx[q * k + o] = wt;
            out_d[q * k + o] = sqrt(wk);
        }
    }
}

}  // namespace mg

using namespace mg;

template <int DIM, int KPL>
static int launch_knn_t(unsigned blocks, size_t, cudaStream_t st, const KnnArgs &a) {
    const size_t smem = sizeof(KnnSmem<KPL>) * kKnnWarps;
    MG_CUDA(cudaFuncSetAttribute(k_knn_hsml<DIM, KPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_knn_hsml<DIM, KPL><<<blocks, kKnnWarps * 32, smem, st>>>(a);
    return MG_OK;
}

template <int DIM>
static int launch_knn_d(int kpl, unsigned blocks, size_t smem, cudaStream_t st, const KnnArgs &a) {
    if (kpl == 1) return launch_knn_t<DIM, 1>(blocks, smem, st, a);
    if (kpl == 2) return launch_knn_t<DIM, 2>(blocks, smem, st, a);
    return launch_knn_t<DIM, 4>(blocks, smem, st, a);
}

template <int DIM>
static int launch_heavy_d(int kpl, unsigned blocks, cudaStream_t st, const KnnArgs &a) {
    if (kpl == 1)
        k_knn_heavy<DIM, 1><<<blocks, kHeavyThreads, 0, st>>>(a);
    else if (kpl == 2)
        k_knn_heavy<DIM, 2><<<blocks, kHeavyThreads, 0, st>>>(a);
    else
        k_knn_heavy<DIM, 4><<<blocks, kHeavyThreads, 0, st>>>(a);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

static int launch_heavy(int dim, int kpl, unsigned blocks, cudaStream_t st, const KnnArgs &a) {
    if (dim == 1) return launch_heavy_d<1>(kpl, blocks, st, a);
    if (dim == 2) return launch_heavy_d<2>(kpl, blocks, st, a);
    return launch_heavy_d<3>(kpl, blocks, st, a);
}

#ifndef MG_KNN_GROUP_G
#define MG_KNN_GROUP_G 128
#endif
#ifndef MG_KNN_GROUP_C
#define MG_KNN_GROUP_C 2048
#endif
constexpr int kGroupThreads = MG_KNN_GROUP_G;  // queries per block of the first pass
constexpr int kGroupStage = MG_KNN_GROUP_C;    // staged candidates per block

template <int DIM>
static int launch_group_d(unsigned blocks, cudaStream_t st, const KnnArgs &a) {
    const size_t smem = sizeof(GroupSmem<kGroupThreads, kGroupStage>);
    MG_CUDA(cudaFuncSetAttribute(k_knn_group<DIM, kGroupThreads, kGroupStage>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_knn_group<DIM, kGroupThreads, kGroupStage><<<blocks, kGroupThreads, smem, st>>>(a);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

static int launch_group(int dim, unsigned blocks, cudaStream_t st, const KnnArgs &a) {
    if (dim == 1) return launch_group_d<1>(blocks, st, a);
    if (dim == 2) return launch_group_d<2>(blocks, st, a);
    return launch_group_d<3>(blocks, st, a);
}

// process-wide switch of the first (group) pass; atomic so that a call on
// one host thread may flip it while another thread launches searches
static std::atomic<int> g_group_pass{1};

extern "C" int mg_knn_set_group_pass(int32_t enabled) {
    return g_group_pass.exchange(enabled ? 1 : 0);
}

// process-wide switch of the cooperative launch of the warp passes; off (the
// default): the host loop of one launch per kernel and pass.  Measured on a
// GB300, the cooperative launch gives the same answers; the search + h stage
// of 2^22 Plummer takes the same time either way (10.72-10.85 against
// 10.78-10.83 ms over two runs), of the 2^24 clump mixture longer (74.6-75.7
// against 72.1-73.4 ms: one wave of resident blocks balances the queue worse
// than two), and a grid that holds every SM keeps the snapshot lanes of a
// batch from overlapping (64 snapshots: 271 against 207 ms).
static std::atomic<int> g_persistent_passes{0};

extern "C" int mg_knn_set_persistent_passes(int32_t enabled) {
    return g_persistent_passes.exchange(enabled ? 1 : 0);
}

// Passes 1 .. pq.npass - 1 in one cooperative launch (k_knn_passes), one wave
// of the blocks the SMs hold at once; done = false when the device cannot
// take it (no cooperative launch, no resident block), and the caller runs the
// host loop instead.
template <int DIM, int KPL>
static int launch_passes_t(int nsm, cudaStream_t st, const KnnArgs &a, const PassQueues &pq, bool &done) {
    done = false;
    const size_t smem = std::max(sizeof(KnnSmem<KPL>) * kKnnWarps, sizeof(HeavySmem<KPL>));
    auto fn = k_knn_passes<DIM, KPL>;
    MG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kKnnWarps * 32, smem));
    if (per_sm < 1) return MG_OK;
    KnnArgs aa = a;
    PassQueues qq = pq;
    void *args[] = {&aa, &qq};
    MG_CUDA(cudaLaunchCooperativeKernel((const void *)fn, dim3((unsigned)(nsm * per_sm)), dim3(kKnnWarps * 32), args,
                                        smem, st));
    done = true;
    return MG_OK;
}

template <int DIM>
static int launch_passes_d(int kpl, int nsm, cudaStream_t st, const KnnArgs &a, const PassQueues &pq, bool &done) {
    if (kpl == 1) return launch_passes_t<DIM, 1>(nsm, st, a, pq, done);
    if (kpl == 2) return launch_passes_t<DIM, 2>(nsm, st, a, pq, done);
    return launch_passes_t<DIM, 4>(nsm, st, a, pq, done);
}

static int launch_passes(int dim, int kpl, int nsm, cudaStream_t st, const KnnArgs &a, const PassQueues &pq,
                         bool &done) {
    done = false;
    int dev = 0, coop = 0;
    MG_CUDA(cudaGetDevice(&dev));
    MG_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop || !g_persistent_passes.load()) return MG_OK;
    if (dim == 1) return launch_passes_d<1>(kpl, nsm, st, a, pq, done);
    if (dim == 2) return launch_passes_d<2>(kpl, nsm, st, a, pq, done);
    return launch_passes_d<3>(kpl, nsm, st, a, pq, done);
}

static int launch_knn(int dim, int kpl, unsigned blocks, size_t smem, cudaStream_t st, const KnnArgs &a) {
    if (dim == 1) return launch_knn_d<1>(kpl, blocks, smem, st, a);
    if (dim == 2) return launch_knn_d<2>(kpl, blocks, smem, st, a);
    return launch_knn_d<3>(kpl, blocks, smem, st, a);
}

static inline CellIndex make_index(const mg_cells *c) {
    CellIndex ci;
    ci.Lg = c->grid_level;
    ci.keys = c->keys;
    ci.cs = c->cell_start;
    const bool use_bricks = c->brick_of && c->bricks && c->brick_capacity > 0;
    ci.brick_of = use_bricks ? c->brick_of : nullptr;
    ci.bricks = use_bricks ? c->bricks : nullptr;
    return ci;
}

static inline void fill_args(KnnArgs &a, const mg_cells *c) {
    a.ci = make_index(c);
    a.n = c->n;
    a.dim = c->dim;
    a.Lg = c->grid_level;
    a.periodic = c->boxsize > 0;
    a.box_hi = (float)c->boxsize;
    a.box64 = c->boxsize;
    a.box_lo = (float)(c->boxsize - (double)a.box_hi);
    a.frame = c->frame;
    a.keys = c->keys;
    a.cell_start = c->cell_start;
    a.order = c->order;
    a.hi = reinterpret_cast<const float4 *>(c->pos_hi);
    a.lo = reinterpret_cast<const float4 *>(c->pos_lo);
    a.pos64 = c->pos64;
}

static inline int64_t heavy_capacity(int64_t nq) { return nq < kHeavyCap ? nq : kHeavyCap; }

extern "C" size_t mg_knn_hsml_workspace_bytes(int64_t nq, int32_t k) {
    if (nq <= 0 || k < 1) return 0;
    // the selected-distance rows are scratch of the h solve only for k > 32
    const size_t dsel_entries = k > 32 ? (size_t)nq * (size_t)k : 0;
    return 3 * align_up(sizeof(float) * nq) + 2 * align_up(sizeof(int32_t) * nq) +
           align_up(sizeof(float) * dsel_entries) +
           align_up(sizeof(int32_t) * (size_t)heavy_capacity(nq) * kHeavyItem) + 3 * align_up(sizeof(int32_t) * 64) +
           1024;
}

extern "C" int mg_knn_hsml(const mg_cells *c, const int32_t *queries, int64_t nq, int32_t k,
                           const float *seed_h, float radius_factor, int32_t level_bias,
                           int32_t max_passes, int32_t *ngb,
                           float *hsml, float *hsml_lo, int32_t *qstatus, int64_t *stats, void *workspace,
                           size_t workspace_bytes, void *stream_) {
    if (!c || nq <= 0 || !seed_h || !ngb || !hsml || !qstatus || !stats) return MG_ERR_ARG;
    if (k < 1 || k > MG_MAX_K) return MG_ERR_UNSUPPORTED;
    if (k > c->n) return MG_ERR_ARG;
    if (max_passes < 1) max_passes = 1;
    if (workspace_bytes < mg_knn_hsml_workspace_bytes(nq, k)) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    Carve w(workspace, workspace_bytes);
    float *radius = w.take<float>(nq);
    float *rlo = w.take<float>(nq);
    float *rhi = w.take<float>(nq);
    int32_t *qa = w.take<int32_t>(nq);
    int32_t *qb = w.take<int32_t>(nq);
    int32_t *counts = w.take<int32_t>(64);
    float *dsel = w.take<float>(k > 32 ? (size_t)nq * (size_t)k : 0);
    const int64_t hcap = heavy_capacity(nq);
    int32_t *heavy = w.take<int32_t>((size_t)hcap * kHeavyItem);
    int32_t *hcounts = w.take<int32_t>(64);
    int32_t *hnext = w.take<int32_t>(64);
    if (!w.ok()) return MG_ERR_ARG;
    MG_CUDA(cudaMemsetAsync(counts, 0, sizeof(int32_t) * 64, st));
    MG_CUDA(cudaMemsetAsync(hcounts, 0, sizeof(int32_t) * 64, st));
    MG_CUDA(cudaMemsetAsync(hnext, 0, sizeof(int32_t) * 64, st));
    MG_CUDA(cudaMemsetAsync(qstatus, 0, sizeof(int32_t) * nq, st));
    KnnArgs a;
    fill_args(a, c);
    a.queries = queries;
    a.nq = nq;
    a.k = k;
    a.seed_h = seed_h;
    a.radius_factor = radius_factor;
    a.level_bias = level_bias < 0 ? 0 : (level_bias > 1 ? 1 : level_bias);  // <= 5 cells per axis
    a.radius = radius;
    a.rlo = rlo;
    a.rhi = rhi;
    a.ngb = ngb;
    a.hsml = hsml;
    a.qstatus = qstatus;
    a.stats = stats;
    a.heavy = heavy;
    a.heavy_cap = (int)hcap;
    int dev = 0, nsm = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    // first pass one thread per query over block-shared candidates (not for
    // periodic boxes or k > 32; its leftovers need a second pass)
    const bool group_first = g_group_pass.load() && !a.periodic && k <= 32 && max_passes >= 2;
    const int kpl = k <= 32 ? 1 : (k <= 64 ? 2 : 4);
    const int npass = std::min(max_passes, 63);
    for (int pass = 0; pass < npass; ++pass) {
        if (pass == 1) {
            // the remaining passes in one cooperative launch where possible
            PassQueues pq{qa, qb, counts, hcounts, hnext, npass, max_passes};
            bool done = false;
            const int rc = launch_passes(c->dim, kpl, nsm, st, a, pq, done);
            if (rc) return rc;
            if (done) {
                MG_CHECK_LAUNCH();
                break;
            }
        }
        a.qin = pass == 0 ? nullptr : (pass % 2 ? qa : qb);
        a.qin_count = pass == 0 ? nullptr : counts + (pass - 1);
        a.qout = pass % 2 ? qb : qa;
        a.qout_count = counts + pass;
        a.last_pass = pass == max_passes - 1;
        a.heavy_count = hcounts + pass;
        a.heavy_next = hnext + pass;
        int64_t blocks;
        if (pass == 0)
            blocks = (nq + kKnnWarps * kChunk - 1) / (kKnnWarps * kChunk);
        else
            blocks = (int64_t)nsm * 8;  // persistent sweep over the queue
        if (blocks > 2147483647) blocks = 2147483647;
        if (pass > 0) k_count_pass<<<1, 32, 0, st>>>(counts + (pass - 1), stats);
        if (pass == 0 && group_first) {
            const int rc = launch_group(c->dim, (unsigned)((nq + kGroupThreads - 1) / kGroupThreads), st, a);
            if (rc) return rc;
            continue;
        }
        const size_t smem = 0;
        int rc = launch_knn(c->dim, kpl, (unsigned)blocks, smem, st, a);
        if (rc) return rc;
        MG_CHECK_LAUNCH();
        rc = launch_heavy(c->dim, kpl, (unsigned)nsm * 4, st, a);
        if (rc) return rc;
    }
    if (c->dim == 1) return launch_hsml_rows<1>(st, a, qstatus, nq, k, dsel, hsml, hsml_lo, stats);
    if (c->dim == 2) return launch_hsml_rows<2>(st, a, qstatus, nq, k, dsel, hsml, hsml_lo, stats);
    return launch_hsml_rows<3>(st, a, qstatus, nq, k, dsel, hsml, hsml_lo, stats);
}

extern "C" int mg_hsml_solve(const float *d2, int64_t nq, int32_t k, int32_t dim, float *hsml, int64_t *stats,
                             void *stream_) {
    if (!d2 || !hsml || nq <= 0 || k < 2 || dim < 1 || dim > 3) return MG_ERR_ARG;
    if (k > MG_MAX_K) return MG_ERR_UNSUPPORTED;
    cudaStream_t st = as_stream(stream_);
    const unsigned hb = (unsigned)((nq + 127) / 128);
    if (dim == 1)
        launch_hsml_solve<1>(hb, st, d2, nullptr, nq, k, hsml, stats);
    else if (dim == 2)
        launch_hsml_solve<2>(hb, st, d2, nullptr, nq, k, hsml, stats);
    else
        launch_hsml_solve<3>(hb, st, d2, nullptr, nq, k, hsml, stats);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" int mg_seed_plain(const mg_cells *c, const int32_t *queries, int64_t nq, int32_t k,
                             float *seed_h, void *stream_) {
    if (!c || nq <= 0 || !seed_h || k < 1) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    k_seed_plain<<<(unsigned)((nq + 255) / 256), 256, 0, st>>>(make_index(c), c->n, c->frame, queries, nq, k,
                                                                  c->dim, seed_h);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" int mg_seed_features(const mg_cells *c, const int32_t *queries, int64_t nq, int32_t k,
                                uint16_t *features, float *cell_side, void *stream_) {
    if (!c || nq <= 0 || !features || !cell_side || k < 1) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    int64_t blocks = (nq + 8 * 32 - 1) / (8 * 32);  // ~32 consecutive queries per warp
    k_seed_features<<<(unsigned)blocks, 256, 0, st>>>(make_index(c), c->n, c->frame, queries, nq, k, c->dim,
                                                                c->boxsize > 0 ? 1 : 0, features,
                                                                cell_side);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" int mg_density(const int32_t *out_rows, const float *hsml, const float *hsml_lo, int64_t nq,
                          const double *m_rows, int32_t des_ngb, int32_t dim, double *h_out, double *density,
                          double *vol, void *stream_) {
    if (nq <= 0 || !hsml || !h_out || dim < 1 || dim > 3 || des_ngb < 1) return MG_ERR_ARG;
    const double pi = 3.14159265358979323846;
    const double volnorm = dim == 1 ? 2.0 : (dim == 2 ? pi : 4.0 * pi / 3.0);
    k_density<<<(unsigned)((nq + 255) / 256), 256, 0, as_stream(stream_)>>>(out_rows, hsml, hsml_lo, nq, m_rows,
                                                                           (double)des_ngb, 1.0 / (double)des_ngb,
                                                                           dim, volnorm, h_out,
                                                                           density, vol);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" int mg_neighbor_dist(const mg_cells *c, const int32_t *queries, int64_t nq,
                                const int32_t *ngb, int32_t k, int64_t *ngb_particles, double *dist,
                                void *stream_) {
    if (!c || nq <= 0 || !ngb || !ngb_particles || !dist) return MG_ERR_ARG;
    if (k < 1 || k > MG_MAX_K) return MG_ERR_UNSUPPORTED;
    cudaStream_t st = as_stream(stream_);
    k_neighbor_dist<<<(unsigned)((nq + 7) / 8), 256, 0, st>>>(c->pos64, c->order, queries, nq, ngb, k,
                                                                c->boxsize > 0, c->boxsize,
                                                                ngb_particles, dist);
    MG_CHECK_LAUNCH();
    return MG_OK;
}
