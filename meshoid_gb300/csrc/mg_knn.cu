// Neighbour search + smoothing-length solve (one warp per query), the plain
// seed, and the per-row FP64 distance accessor.
//
// Replaces cKDTree.query(pos[mask], des_ngb) (src/meshoid/Meshoid.py:157)
// followed by HsmlIter (src/meshoid/kernel_density.py:15-56).
//
// Search: the query's first radius R comes from a seed.  The level L with
// cell side s_L >= R is chosen, the (at most 27) level-L cells that meet the
// sphere of radius R are looked up (dense table for L <= grid_level, binary
// search of the Morton keys below), and every particle of those cells with
// FP32 d^2 <= R^2 is appended to a per-warp shared-memory buffer.  Fewer than
// k hits, or more than the buffer holds, re-queues the query with a corrected
// radius (work queue over passes).  The k smallest are picked by a 32-bucket
// histogram in (d/R)^dim; entries within 1e-5 (relative, in d^2) of the k-th
// distance are re-decided with exact FP64 distances and the particle index,
// so the set equals the k smallest by (FP64 d^2, index).
//
// h: norm * sum_j W(d_j/h) = k (norm = 32/3, 40/7, 8/3 in 3/2/1-D), solved by
// bracketed Newton (bisection fallback) on the k distances held across the
// warp.  The function is C^2 and increasing in h, so the root is unique; the
// reference bisects to |n - k| <= 1e-13 and outputs the midpoint, i.e. the
// same root.
#include <cfloat>

#include "mg_common.cuh"

namespace mg {

constexpr int kKnnWarps = 8;     // warps per block
constexpr int kKnnCap = 512;     // candidate buffer per warp
constexpr float kBandEps = 1e-5f;
constexpr int kMaxCellsPerQuery = 125;

struct KnnArgs {
    int64_t n;
    int dim, Lg;
    bool periodic;
    float box_hi, box_lo;
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
};

__device__ __forceinline__ uint32_t lower_bound_prefix(const uint64_t *__restrict__ keys, uint32_t a,
                                                       uint32_t b, uint64_t code, int ks) {
    while (a < b) {
        uint32_t m = a + ((b - a) >> 1);
        if ((keys[m] >> ks) < code)
            a = m + 1;
        else
            b = m;
    }
    return a;
}

// Slot range [a, b) of the level-L cell with coordinates (cx, cy, cz).
__device__ __forceinline__ void cell_range(int L, int Lg, uint32_t cx, uint32_t cy, uint32_t cz,
                                           const uint64_t *__restrict__ keys,
                                           const uint32_t *__restrict__ cs, uint32_t &a,
                                           uint32_t &b) {
    const uint64_t code = morton3(cx, cy, cz);
    if (L <= Lg) {
        const int sh = 3 * (Lg - L);
        a = __ldg(cs + (code << sh));
        b = __ldg(cs + ((code + 1) << sh));
    } else {
        const uint64_t anc = code >> (3 * (L - Lg));
        const uint32_t A = __ldg(cs + anc), B = __ldg(cs + anc + 1);
        const int ks = 3 * (kKeyBits - L);
        a = lower_bound_prefix(keys, A, B, code, ks);
        b = lower_bound_prefix(keys, a, B, code + 1, ks);
    }
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

template <int DIM>
__global__ __launch_bounds__(kKnnWarps * 32) void k_knn_hsml(KnnArgs a) {
    __shared__ float s_d[kKnnWarps][kKnnCap];
    __shared__ int32_t s_i[kKnnWarps][kKnnCap];
    __shared__ int32_t s_hist[kKnnWarps][32];
    __shared__ float s_sel[kKnnWarps][MG_MAX_K];
    __shared__ uint32_t s_ca[kKnnWarps][32], s_cb[kKnnWarps][32];

    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float *bd = s_d[wib];
    int32_t *bi = s_i[wib];
    const int64_t gwarp = (int64_t)blockIdx.x * kKnnWarps + wib;
    const int64_t nwarps = (int64_t)gridDim.x * kKnnWarps;
    const int64_t count = a.qin ? (int64_t)*a.qin_count : a.nq;
    const Frame fr = load_frame(a.frame);
    const float side = (float)fr.side;
    const float half_side = 0.5f * side;
    const int k = a.k;
    const float norm = DIM == 3 ? 32.0f / 3.0f : (DIM == 2 ? 40.0f / 7.0f : 8.0f / 3.0f);
    const float bound_coeff = 1.0f / (1.0f - powf(2.0f * norm, -1.0f / 3.0f));

    int64_t st_cand = 0, st_retry = 0, st_band = 0, st_unres = 0, st_newton = 0;
    int64_t st_reason[3] = {0, 0, 0};
    int32_t my_retry = -1;  // lane i holds the i-th pending retry of this warp
    int n_retry = 0;

    for (int64_t item = gwarp; item < count; item += nwarps) {
        const int32_t qi = a.qin ? a.qin[item] : (int32_t)item;
        const int32_t p = a.queries ? a.queries[qi] : qi;
        float R = a.qin ? a.radius[qi] : a.seed_h[qi] * a.radius_factor;
        if (!(R > 0.0f) || !isfinite(R)) R = side * 1e-3f;
        const float4 h0 = a.hi[p], l0 = a.lo[p];

        // ---- level and cell box ------------------------------------------
        int L = (int)floorf(log2f(side / R)) + a.level_bias;
        L = max(0, min(kMaxLevel, L));
        const float cells_per_side = (float)(1u << L);
        const float scale = cells_per_side / side;
        const float u[3] = {((h0.x + half_side) + l0.x) * scale, ((h0.y + half_side) + l0.y) * scale,
                            ((h0.z + half_side) + l0.z) * scale};
        const float rc = R * scale * (1.0f + 1e-5f) + 1e-3f + cells_per_side * 2.4e-7f;
        int cmin[3], cnum[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
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
                }
            } else {
                lo_c = max(lo_c, 0);
                hi_c = min(hi_c, (int)cells_per_side - 1);
            }
            cmin[d] = lo_c;
            cnum[d] = max(0, hi_c - lo_c + 1);
        }
        // level_bias <= 1 bounds the box to 5 cells per axis (125 cells)
        const int ncell = cnum[0] * cnum[1] * cnum[2];
        const float R2 = R * R;

        // ---- gather candidates with d^2 <= R^2 -----------------------------
        // mode 0 fills the buffer; mode 1 (only after an overflow) re-scans the
        // same cells and histograms all in-radius candidates so the next radius
        // can be cut to the bucket that holds the k-th neighbour.
        int cnt = 0;
        const float invR2 = 1.0f / R2;
        // histogram window in v = (d/R)^DIM: [v_lo, v_lo + 32 v_w), c_below
        // in-radius candidates lie under v_lo
        float v_lo = 0.0f, v_w = 1.0f / 32.0f, v_hi = 1.0f;
        int c_below = 0;
        bool overflow_done = false;
        for (int mode = 0; mode < 4; ++mode) {
            if (mode >= 1) {
                if (cnt <= kKnnCap || overflow_done) break;
                s_hist[wib][lane] = 0;
                __syncwarp();
            }
            for (int cb = 0; cb < ncell; cb += 32) {
                const int c = cb + lane;
                uint32_t ca = 0, cbnd = 0;
                if (c < ncell) {
                    int ix = c % cnum[0], iy = (c / cnum[0]) % cnum[1], iz = c / (cnum[0] * cnum[1]);
                    int gx = cmin[0] + ix, gy = cmin[1] + iy, gz = cmin[2] + iz;
                    // sphere-box test in cell units
                    float dx = fmaxf(0.0f, fmaxf((float)gx - u[0], u[0] - (float)(gx + 1)));
                    float dy = fmaxf(0.0f, fmaxf((float)gy - u[1], u[1] - (float)(gy + 1)));
                    float dz = fmaxf(0.0f, fmaxf((float)gz - u[2], u[2] - (float)(gz + 1)));
                    if (DIM < 3) dz = 0.0f;
                    if (DIM < 2) dy = 0.0f;
                    if (dx * dx + dy * dy + dz * dz <= rc * rc) {
                        const int M = (int)cells_per_side;
                        if (a.periodic) {
                            gx = ((gx % M) + M) % M;
                            gy = ((gy % M) + M) % M;
                            gz = ((gz % M) + M) % M;
                        }
                        if (DIM < 3) gz = 0;
                        if (DIM < 2) gy = 0;
                        cell_range(L, a.Lg, (uint32_t)gx, (uint32_t)gy, (uint32_t)gz, a.keys, a.cell_start,
                                   ca, cbnd);
                    }
                }
                s_ca[wib][lane] = ca;
                s_cb[wib][lane] = cbnd;
                unsigned nonempty = __ballot_sync(0xffffffffu, cbnd > ca);
                __syncwarp();
                while (nonempty) {
                    const int j = __ffs(nonempty) - 1;
                    nonempty &= nonempty - 1;
                    const uint32_t A = s_ca[wib][j], B = s_cb[wib][j];
                    for (uint32_t t0 = A; t0 < B; t0 += 32) {
                        const uint32_t t = t0 + lane;
                        float dd = FLT_MAX;
                        if (t < B) {
                            const float4 hb = a.hi[t], lb = a.lo[t];
                            float3 s = a.periodic ? sep_hilo_periodic(h0, l0, hb, lb, a.box_hi, a.box_lo)
                                                  : sep_hilo(h0, l0, hb, lb);
                            dd = s.x * s.x + s.y * s.y + s.z * s.z;
                        }
                        const bool in = dd <= R2;
                        if (mode == 0) {
                            const unsigned m = __ballot_sync(0xffffffffu, in);
                            const int pos = cnt + __popc(m & ((1u << lane) - 1u));
                            if (in && pos < kKnnCap) {
                                bd[pos] = dd;
                                bi[pos] = (int32_t)t;
                            }
                            cnt += __popc(m);
                        } else if (in) {
                            const float t = dd * invR2;
                            const float v = DIM == 3 ? t * sqrtf(t) : (DIM == 2 ? t : sqrtf(t));
                            if (v >= v_lo && v < v_hi)
                                atomicAdd(&s_hist[wib][min(31, (int)((v - v_lo) / v_w))], 1);
                        }
                        st_cand += (t0 + 32 <= B) ? 32 : (int64_t)(B - t0);
                    }
                }
                __syncwarp();
            }
            __syncwarp();
            if (mode >= 1) {
                // locate the sub-bucket holding the k-th and narrow the window
                const int hc = s_hist[wib][lane];
                const int cum = warp_incl_scan(hc) + c_below;
                const int bk = __ffs(__ballot_sync(0xffffffffu, cum >= k)) - 1;
                const int cum_bk = __shfl_sync(0xffffffffu, cum, max(bk, 0));
                const int hc_bk = __shfl_sync(0xffffffffu, hc, max(bk, 0));
                if (bk < 0) {  // numerical edge: keep the window
                    overflow_done = true;
                } else {
                    v_hi = v_lo + (float)(bk + 1) * v_w;
                    if (cum_bk <= kKnnCap) {
                        overflow_done = true;
                    } else {
                        c_below = cum_bk - hc_bk;
                        v_lo = v_lo + (float)bk * v_w;
                        v_w = v_w / 32.0f;
                    }
                }
            }
        }

        // ---- too few / too many: re-queue with a corrected radius ----------
        float Rnew = -1.0f;
        int reason = 0;
        if (cnt < k) {
            float g = 1.25f * powf((float)k / (float)max(cnt, 1), 1.0f / DIM);
            Rnew = R * fminf(fmaxf(g, 1.25f), 4.0f);
            reason = 1;
        } else if (cnt > kKnnCap) {
            // shrink to the upper edge of the histogram window holding the k-th
            Rnew = R * (DIM == 3 ? cbrtf(v_hi) : (DIM == 2 ? sqrtf(v_hi) : v_hi)) * 1.00001f;
            if (Rnew >= R) Rnew = R * 0.999f;
            reason = 2;
        }

        // ---- select the k smallest: bucket histogram ------------------------
        float T = 0.0f;
        int b_star = 0, c_lo = 0;
        if (Rnew < 0.0f) {
            s_hist[wib][lane] = 0;
            __syncwarp();
            for (int e = lane; e < cnt; e += 32) atomicAdd(&s_hist[wib][(int)bucket_of(bd[e] * invR2, DIM)], 1);
            __syncwarp();
            const int hcount = s_hist[wib][lane];
            const int cum = warp_incl_scan(hcount);
            b_star = __ffs(__ballot_sync(0xffffffffu, cum >= k)) - 1;
            const int cum_b = __shfl_sync(0xffffffffu, cum, b_star);
            const int m_b = __shfl_sync(0xffffffffu, hcount, b_star);
            c_lo = cum_b - m_b;
            const int r = k - c_lo;
            int32_t *row = a.ngb + (int64_t)qi * k;
            // sure part: buckets below b_star
            int out = 0, nb = 0;
            for (int e0 = 0; e0 < cnt; e0 += 32) {
                const int e = e0 + lane;
                float v = e < cnt ? bd[e] : FLT_MAX;
                int bk = e < cnt ? (int)bucket_of(v * invR2, DIM) : 99;
                const bool sure = bk < b_star;
                unsigned ms = __ballot_sync(0xffffffffu, sure);
                if (sure) {
                    int pos = out + __popc(ms & ((1u << lane) - 1u));
                    row[pos] = bi[e];
                    s_sel[wib][pos] = v;
                }
                out += __popc(ms);
                const bool bnd = bk == b_star;
                unsigned mb = __ballot_sync(0xffffffffu, bnd);
                if (bnd && m_b <= 32) {
                    int pos = nb + __popc(mb & ((1u << lane) - 1u));
                    s_ca[wib][pos] = __float_as_uint(v);
                    s_cb[wib][pos] = (uint32_t)bi[e];
                }
                nb += __popc(mb);
            }
            __syncwarp();
            if (m_b <= 32) {
                float key = lane < m_b ? __uint_as_float(s_ca[wib][lane]) : FLT_MAX;
                int32_t tie = lane < m_b ? (int32_t)s_cb[wib][lane] : INT_MAX;
                warp_sort_pairs(key, tie);
                if (lane < r) {
                    row[c_lo + lane] = tie;
                    s_sel[wib][c_lo + lane] = key;
                }
                T = __shfl_sync(0xffffffffu, key, r - 1);
            } else {
                // many entries share the boundary bucket: take the r smallest one
                // at a time (rare: heavy exact/near ties)
                for (int rep = 0; rep < r; ++rep) {
                    float best = FLT_MAX;
                    int32_t bslot = INT_MAX;
                    int bidx = -1;
                    for (int e = lane; e < cnt; e += 32) {
                        if ((int)bucket_of(bd[e] * invR2, DIM) != b_star || bi[e] < 0) continue;
                        if (bd[e] < best || (bd[e] == best && bi[e] < bslot)) {
                            best = bd[e];
                            bslot = bi[e];
                            bidx = e;
                        }
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        float ob = __shfl_xor_sync(0xffffffffu, best, o);
                        int32_t os = __shfl_xor_sync(0xffffffffu, bslot, o);
                        int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
                        if (ob < best || (ob == best && os < bslot)) {
                            best = ob;
                            bslot = os;
                            bidx = oi;
                        }
                    }
                    if (lane == 0) {
                        row[c_lo + rep] = bslot;
                        s_sel[wib][c_lo + rep] = best;
                        bi[bidx] = -1 - bslot;  // mark taken
                    }
                    __syncwarp();
                    T = best;
                }
                for (int e = lane; e < cnt; e += 32)
                    if (bi[e] < 0) bi[e] = -1 - bi[e];
            }
            __syncwarp();
            // the band around T must lie inside the searched radius
            if (T * (1.0f + kBandEps) > R2) {
                Rnew = sqrtf(T * (1.0f + 2.0f * kBandEps)) * 1.0001f;
                reason = 3;
            }
        }

        if (Rnew > 0.0f) {
            st_reason[reason - 1] += 1;
            if (a.last_pass) {
                if (lane == 0) {
                    a.qstatus[qi] |= MG_Q_UNRESOLVED;
                    // diagnostics for the caller: last radius and candidate count
                    a.radius[qi] = R;
                    a.hsml[qi] = -(float)(cnt + 1000000 * reason);
                }
                st_unres += 1;
            } else {
                if (lane == 0) a.radius[qi] = Rnew;
                if (lane == n_retry) my_retry = qi;
                ++n_retry;
                st_retry += 1;
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

        // ---- FP64 re-decision of the band around the k-th distance --------
        const float lo_band = T * (1.0f - kBandEps), hi_band = T * (1.0f + kBandEps);
        int nband = 0;
        for (int e0 = 0; e0 < cnt; e0 += 32) {
            const int e = e0 + lane;
            const bool inb = e < cnt && bd[e] >= lo_band && bd[e] <= hi_band;
            nband += __popc(__ballot_sync(0xffffffffu, inb));
        }
        int32_t *row = a.ngb + (int64_t)qi * k;
        if (nband > 1) {
            st_band += 1;
            // gather band members (at most 32 resolved exactly; more is flagged)
            int nb = 0, nsure = 0;
            for (int e0 = 0; e0 < cnt; e0 += 32) {
                const int e = e0 + lane;
                const bool inb = e < cnt && bd[e] >= lo_band && bd[e] <= hi_band;
                const bool sure = e < cnt && bd[e] < lo_band;
                unsigned mb = __ballot_sync(0xffffffffu, inb);
                unsigned ms = __ballot_sync(0xffffffffu, sure);
                if (inb) {
                    int pos = nb + __popc(mb & ((1u << lane) - 1u));
                    if (pos < 32) s_cb[wib][pos] = (uint32_t)bi[e];
                }
                if (sure) {
                    int pos = nsure + __popc(ms & ((1u << lane) - 1u));
                    row[pos] = bi[e];
                    s_sel[wib][pos] = bd[e];
                }
                nb += __popc(mb);
                nsure += __popc(ms);
            }
            __syncwarp();
            const int need = k - nsure;
            double key = DBL_MAX;
            int32_t tie = INT_MAX;
            int32_t slot = -1;
            if (lane < min(nb, 32)) {
                slot = (int32_t)s_cb[wib][lane];
                key = d2_exact(a.pos64, p, slot, a.periodic, fr.side);
                tie = a.order[slot];
            }
            // sort by (FP64 d2, particle index); carry the slot through a shuffle
            // of the particle index -> slot map kept alongside
            int32_t carry = slot;
            {
#pragma unroll
                for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
                    for (int stride = size >> 1; stride > 0; stride >>= 1) {
                        double okey = __shfl_xor_sync(0xffffffffu, key, stride);
                        int32_t otie = __shfl_xor_sync(0xffffffffu, tie, stride);
                        int32_t ocar = __shfl_xor_sync(0xffffffffu, carry, stride);
                        const bool up = ((lane & size) == 0);
                        const bool lower = ((lane & stride) == 0);
                        const bool other_less = (okey < key) || (okey == key && otie < tie);
                        const bool same = (okey == key && otie == tie);
                        const bool take = (lower == up) ? other_less : (!other_less && !same);
                        if (take) {
                            key = okey;
                            tie = otie;
                            carry = ocar;
                        }
                    }
                }
            }
            if (lane >= nb) carry = p;  // never hand out an invalid slot (flagged below)
            if (lane < need) {
                row[nsure + lane] = carry;
                s_sel[wib][nsure + lane] = (float)key;
            }
            if (nb > 32 || need > 32 || need > nb) {
                if (lane == 0) {
                    a.qstatus[qi] |= MG_Q_UNRESOLVED;
                    a.hsml[qi] = -(float)(nb + 4000000);
                }
                st_unres += 1;
                st_reason[2] += 1000000;
                continue;
            }
            if (lane == 0) a.qstatus[qi] |= MG_Q_BAND_FP64;
            __syncwarp();
        }

        // ---- smoothing length ----------------------------------------------
        const int kpl = (k + 31) >> 5;
        float dist[MG_MAX_K / 32];
        float dmin = FLT_MAX, dmax = 0.0f;
#pragma unroll
        for (int j = 0; j < MG_MAX_K / 32; ++j) {
            const int e = lane + 32 * j;
            dist[j] = (j < kpl && e < k) ? sqrtf(s_sel[wib][e]) : -1.0f;
            if (dist[j] >= 0.0f) dmax = fmaxf(dmax, dist[j]);
        }
        dmax = warp_max(dmax);
        // second-smallest distance (the reference's lower bracket)
        float m1 = FLT_MAX;
#pragma unroll
        for (int j = 0; j < MG_MAX_K / 32; ++j)
            if (dist[j] >= 0.0f) m1 = fminf(m1, dist[j]);
        const float d_min = warp_min(m1);
        float m2 = FLT_MAX;
        {
            bool skipped = false;  // skip one copy of the minimum per lane set
            // count how many lanes hold the minimum; the second smallest equals
            // the minimum when it occurs twice
            int nmin = 0;
#pragma unroll
            for (int j = 0; j < MG_MAX_K / 32; ++j) nmin += (dist[j] == d_min);
            nmin = warp_sum(nmin);
#pragma unroll
            for (int j = 0; j < MG_MAX_K / 32; ++j) {
                if (dist[j] < 0.0f) continue;
                if (dist[j] == d_min && !skipped && nmin == 1) {
                    skipped = true;
                    continue;
                }
                m2 = fminf(m2, dist[j]);
            }
            dmin = warp_min(m2);
        }
        float lower = dmin, upper = dmax * bound_coeff;
        float h = a.seed_h[qi];
        if (!(h > lower && h < upper)) h = 0.5f * (lower + upper);
        const float kf = (float)k;
        int it = 0;
        bool polish = false;
        for (; it < 60; ++it) {
            const float hinv = 1.0f / h;
            float sw = 0.0f, sdw = 0.0f;
#pragma unroll
            for (int j = 0; j < MG_MAX_K / 32; ++j) {
                if (dist[j] < 0.0f) continue;
                const float q = dist[j] * hinv;
                sw += spline_w(q);
                sdw += spline_dw(q) * q;
            }
            sw = warp_sum(sw);
            sdw = warp_sum(sdw);
            const float F = norm * sw - kf;
            const float dF = -norm * sdw * hinv;  // dn/dh >= 0
            // Near the root one further Newton step brings h to the FP32 noise
            // floor of F (~1e-7 relative in h); then stop.
            const bool close = fabsf(F) <= 1e-6f * kf;
            if (F > 0.0f)
                upper = h;
            else
                lower = h;
            float hn = (dF > 0.0f) ? h - F / dF : -1.0f;
            if (!(hn >= lower && hn <= upper)) hn = 0.5f * (lower + upper);
            const bool done = polish || fabsf(hn - h) <= 1e-8f * h || (upper - lower) <= 1e-8f * h;
            h = hn;
            if (done) break;
            polish = close;
        }
        st_newton += it + 1;
        if (lane == 0) a.hsml[qi] = h;
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
        if (st_cand) atomicAdd((unsigned long long *)&a.stats[1], (unsigned long long)st_cand);
        if (st_retry) atomicAdd((unsigned long long *)&a.stats[2], (unsigned long long)st_retry);
        if (st_band) atomicAdd((unsigned long long *)&a.stats[3], (unsigned long long)st_band);
        if (st_unres) atomicAdd((unsigned long long *)&a.stats[4], (unsigned long long)st_unres);
        if (st_newton) atomicAdd((unsigned long long *)&a.stats[5], (unsigned long long)st_newton);
        for (int r = 0; r < 3; ++r)
            if (st_reason[r]) atomicAdd((unsigned long long *)&a.stats[6 + r], (unsigned long long)st_reason[r]);
    }
}

__global__ void k_count_pass(const int32_t *qcount, int64_t *stats) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && *qcount > 0) atomicAdd((unsigned long long *)&stats[0], 1ull);
}

// ---- plain seed --------------------------------------------------------------
// h from the particle count of the query's adaptive cell: the finest level whose
// cell around the query still holds at least max(2, k/4) particles.
__device__ __forceinline__ void own_cell_range(uint64_t key, int L, int Lg,
                                               const uint64_t *__restrict__ keys,
                                               const uint32_t *__restrict__ cs, uint32_t &a,
                                               uint32_t &b) {
    const uint64_t code = key >> (3 * (kKeyBits - L));
    if (L <= Lg) {
        const int sh = 3 * (Lg - L);
        a = __ldg(cs + (code << sh));
        b = __ldg(cs + ((code + 1) << sh));
    } else {
        const uint64_t anc = code >> (3 * (L - Lg));
        const uint32_t A = __ldg(cs + anc), B = __ldg(cs + anc + 1);
        const int ks = 3 * (kKeyBits - L);
        a = lower_bound_prefix(keys, A, B, code, ks);
        b = lower_bound_prefix(keys, a, B, code + 1, ks);
    }
}

__device__ __forceinline__ int adaptive_level(uint64_t key, int Lg, int cmin,
                                              const uint64_t *__restrict__ keys,
                                              const uint32_t *__restrict__ cs, uint32_t &count) {
    uint32_t a, b;
    own_cell_range(key, Lg, Lg, keys, cs, a, b);
    int L = Lg;
    if ((int)(b - a) >= cmin) {
        while (L < kMaxLevel) {
            uint32_t a2, b2;
            own_cell_range(key, L + 1, Lg, keys, cs, a2, b2);
            if ((int)(b2 - a2) < cmin) break;
            a = a2;
            b = b2;
            ++L;
        }
    } else {
        while (L > 0 && (int)(b - a) < cmin) {
            --L;
            own_cell_range(key, L, Lg, keys, cs, a, b);
        }
    }
    count = b - a;
    return L;
}

__global__ void k_seed_plain(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ cs,
                             int Lg, const double *__restrict__ framep, const int32_t *queries,
                             int64_t nq, int k, int dim, float *__restrict__ seed_h) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int32_t p = queries ? queries[q] : (int32_t)q;
    const int cmin = max(2, k / 4);
    uint32_t cnt;
    const int L = adaptive_level(keys[p], Lg, cmin, keys, cs, cnt);
    const float s = (float)(framep[3] / (double)(1u << L));
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
__global__ __launch_bounds__(256) void k_seed_features(const uint64_t *__restrict__ keys,
                                                       const uint32_t *__restrict__ cs, int Lg,
                                                       const double *__restrict__ framep,
                                                       const int32_t *queries, int64_t nq, int k,
                                                       int dim, int periodic,
                                                       uint16_t *__restrict__ feat,
                                                       float *__restrict__ cell_side) {
    const int lane = threadIdx.x & 31;
    const int64_t q = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= nq) return;
    const int32_t p = queries ? queries[q] : (int32_t)q;
    const uint64_t key = keys[p];
    uint32_t cnt = 0;
    int L = 0;
    if (lane == 0) L = adaptive_level(key, Lg, max(2, k / 4), keys, cs, cnt);
    L = __shfl_sync(0xffffffffu, L, 0);
    // integer cell coordinates of the query at level 21
    uint32_t c21[3] = {0, 0, 0};
    for (int b = 0; b < kKeyBits; ++b) {
        c21[0] |= (uint32_t)((key >> (3 * b)) & 1ull) << b;
        c21[1] |= (uint32_t)((key >> (3 * b + 1)) & 1ull) << b;
        c21[2] |= (uint32_t)((key >> (3 * b + 2)) & 1ull) << b;
    }
    float v0 = 0.0f, v1 = 0.0f;
    for (int lev = 0; lev < 2; ++lev) {
        const int LL = max(0, L - lev);
        const int M = 1 << LL;
        float val = 0.0f;
        if (lane < 27) {
            int off[3] = {lane % 3 - 1, (lane / 3) % 3 - 1, lane / 9 - 1};
            int g[3];
            bool ok = true;
            for (int d = 0; d < 3; ++d) {
                g[d] = (int)(c21[d] >> (kKeyBits - LL)) + (d < dim ? off[d] : 0);
                if (d >= dim && off[d] != 0) ok = false;  // collapsed axis
                if (periodic)
                    g[d] = ((g[d] % M) + M) % M;
                else if (g[d] < 0 || g[d] >= M)
                    ok = false;
            }
            if (ok) {
                uint32_t ca, cb;
                cell_range(LL, Lg, (uint32_t)g[0], (uint32_t)g[1], (uint32_t)g[2], keys, cs, ca, cb);
                val = log2f(1.0f + (float)(cb - ca));
            }
        }
        if (lev == 0)
            v0 = val;
        else
            v1 = val;
    }
    // row layout: [0, 27) level L, [27, 54) level L-1, [54, 64) zero
    uint16_t *row = feat + q * MG_MLP_IN_PAD;
    const float vals[2] = {v0, v1};
    for (int h2 = 0; h2 < 2; ++h2) {
        const int idx = lane + 32 * h2;  // 0..63
        float v = 0.0f;
        if (idx < 27)
            v = __shfl_sync(0xffffffffu, vals[0], idx);
        else if (idx < 54)
            v = __shfl_sync(0xffffffffu, vals[1], idx - 27);
        else
            __shfl_sync(0xffffffffu, vals[0], 0);
        // round to bf16 (nearest even)
        uint32_t bits = __float_as_uint(v);
        bits += 0x7fffu + ((bits >> 16) & 1u);
        row[idx] = (uint16_t)(bits >> 16);
    }
    if (lane == 0) cell_side[q] = (float)(framep[3] / (double)(1u << L));
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

static inline void fill_args(KnnArgs &a, const mg_cells *c) {
    a.n = c->n;
    a.dim = c->dim;
    a.Lg = c->grid_level;
    a.periodic = c->boxsize > 0;
    a.box_hi = (float)c->boxsize;
    a.box_lo = (float)(c->boxsize - (double)a.box_hi);
    a.frame = c->frame;
    a.keys = c->keys;
    a.cell_start = c->cell_start;
    a.order = c->order;
    a.hi = reinterpret_cast<const float4 *>(c->pos_hi);
    a.lo = reinterpret_cast<const float4 *>(c->pos_lo);
    a.pos64 = c->pos64;
}

extern "C" size_t mg_knn_hsml_workspace_bytes(int64_t nq) {
    return align_up(sizeof(float) * nq) + 2 * align_up(sizeof(int32_t) * nq) + 1024;
}

extern "C" int mg_knn_hsml(const mg_cells *c, const int32_t *queries, int64_t nq, int32_t k,
                           const float *seed_h, float radius_factor, int32_t level_bias,
                           int32_t max_passes, int32_t *ngb,
                           float *hsml, int32_t *qstatus, int64_t *stats, void *workspace,
                           size_t workspace_bytes, void *stream_) {
    if (!c || nq <= 0 || !seed_h || !ngb || !hsml || !qstatus || !stats) return MG_ERR_ARG;
    if (k < 1 || k > MG_MAX_K) return MG_ERR_UNSUPPORTED;
    if (k > c->n) return MG_ERR_ARG;
    if (max_passes < 1) max_passes = 1;
    if (workspace_bytes < mg_knn_hsml_workspace_bytes(nq)) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    Carve w(workspace, workspace_bytes);
    float *radius = w.take<float>(nq);
    int32_t *qa = w.take<int32_t>(nq);
    int32_t *qb = w.take<int32_t>(nq);
    int32_t *counts = w.take<int32_t>(64);
    if (!w.ok()) return MG_ERR_ARG;
    MG_CUDA(cudaMemsetAsync(counts, 0, sizeof(int32_t) * 64, st));
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
    a.ngb = ngb;
    a.hsml = hsml;
    a.qstatus = qstatus;
    a.stats = stats;
    int dev = 0, nsm = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    for (int pass = 0; pass < max_passes; ++pass) {
        a.qin = pass == 0 ? nullptr : (pass % 2 ? qa : qb);
        a.qin_count = pass == 0 ? nullptr : counts + (pass - 1);
        a.qout = pass % 2 ? qb : qa;
        a.qout_count = counts + pass;
        a.last_pass = pass == max_passes - 1;
        int64_t blocks;
        if (pass == 0)
            blocks = (nq + kKnnWarps - 1) / kKnnWarps;
        else
            blocks = (int64_t)nsm * 8;  // persistent sweep over the queue
        if (blocks > 2147483647) blocks = 2147483647;
        if (pass > 0) k_count_pass<<<1, 32, 0, st>>>(counts + (pass - 1), stats);
        switch (c->dim) {
            case 1: k_knn_hsml<1><<<(unsigned)blocks, kKnnWarps * 32, 0, st>>>(a); break;
            case 2: k_knn_hsml<2><<<(unsigned)blocks, kKnnWarps * 32, 0, st>>>(a); break;
            default: k_knn_hsml<3><<<(unsigned)blocks, kKnnWarps * 32, 0, st>>>(a); break;
        }
        MG_CHECK_LAUNCH();
        if (pass >= 62) break;
    }
    return MG_OK;
}

extern "C" int mg_seed_plain(const mg_cells *c, const int32_t *queries, int64_t nq, int32_t k,
                             float *seed_h, void *stream_) {
    if (!c || nq <= 0 || !seed_h || k < 1) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    k_seed_plain<<<(unsigned)((nq + 255) / 256), 256, 0, st>>>(c->keys, c->cell_start, c->grid_level,
                                                                  c->frame, queries, nq, k, c->dim,
                                                                  seed_h);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" int mg_seed_features(const mg_cells *c, const int32_t *queries, int64_t nq, int32_t k,
                                uint16_t *features, float *cell_side, void *stream_) {
    if (!c || nq <= 0 || !features || !cell_side || k < 1) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    k_seed_features<<<(unsigned)((nq + 7) / 8), 256, 0, st>>>(c->keys, c->cell_start, c->grid_level,
                                                                c->frame, queries, nq, k, c->dim,
                                                                c->boxsize > 0 ? 1 : 0, features,
                                                                cell_side);
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
