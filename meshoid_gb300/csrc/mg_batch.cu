// Many snapshots in one stream-ordered call (mg_batched_run): for each
// snapshot the cell index, plain seed, neighbours + h, first derivatives of its
// fields and its column density map, with every scratch buffer carved from one
// caller workspace and no host synchronisation, so that the whole batch can be
// captured in one CUDA graph.  The reference has no such entry point: its user
// loops over snapshots with one Meshoid each (src/meshoid/Meshoid.py:15-105,
// :237-268, :595-643).
#include <cstring>

#include "mg_common.cuh"

namespace mg {

// Buffers of one snapshot, laid out by the same carve for sizing and running.
struct SnapPlan {
    mg_cells c;
    float *seed, *hsml32, *hsml_lo, *fhi, *flo;
    int32_t *ngb, *qstatus, *gstatus;
    int64_t *stats;
    double *hmap;
    void *ws_build, *ws_knn, *ws_grad, *ws_sd;
    size_t b_build, b_knn, b_grad, b_sd;
};

static size_t plan_snapshot(const mg_snapshot &s, int k, void *base, size_t bytes, SnapPlan &P) {
    Carve w(base, bytes);
    const int64_t n = s.n;
    const int Lg = s.grid_level > 0 ? s.grid_level : mg_default_grid_level(n);
    std::memset(&P, 0, sizeof(P));
    P.c.n = n;
    P.c.dim = 3;
    P.c.grid_level = Lg;
    P.c.boxsize = -1.0;
    P.c.frame = w.take<double>(8);
    P.c.keys = w.take<uint64_t>(n);
    P.c.order = w.take<int32_t>(n);
    P.c.rank = w.take<int32_t>(n);
    P.c.pos_hi = w.take<float>(4 * n);
    P.c.pos_lo = w.take<float>(4 * n);
    P.c.pos64 = w.take<double>(3 * n);
    P.c.cell_start = w.take<uint32_t>(((size_t)1 << (3 * Lg)) + 1);
    if (s.brick_threshold > 0) {
        const int cap = min(mg_brick_capacity(n, Lg, s.brick_threshold), mg_brick_capacity(n, Lg, 64));
        P.c.brick_of = w.take<int32_t>((size_t)1 << (3 * Lg));
        P.c.bricks = w.take<uint32_t>((size_t)cap * MG_BRICK_WORDS);
        P.c.brick_capacity = cap;
        P.c.brick_threshold = s.brick_threshold;
    }
    P.b_build = mg_build_cells_workspace_bytes(n, Lg);
    P.ws_build = w.take<char>(P.b_build);
    P.seed = w.take<float>(n);
    P.hsml32 = w.take<float>(n);
    P.hsml_lo = w.take<float>(n);
    P.ngb = w.take<int32_t>((size_t)n * k);
    P.qstatus = w.take<int32_t>(n);
    P.stats = w.take<int64_t>(16);
    P.b_knn = mg_knn_hsml_workspace_bytes(n, k);
    P.ws_knn = w.take<char>(P.b_knn);
    if (s.nf > 0) {
        const int nfp = (s.nf + 3) & ~3;
        P.fhi = w.take<float>((size_t)n * nfp);
        P.flo = w.take<float>((size_t)n * nfp);
        P.gstatus = w.take<int32_t>(n);
        P.b_grad = mg_grad_sweep_workspace_bytes(n);
        P.ws_grad = w.take<char>(P.b_grad);
    }
    if (s.map) {
        P.hmap = w.take<double>(n);
        P.b_sd = mg_surface_density_workspace_bytes(n, s.map_res);
        P.ws_sd = w.take<char>(P.b_sd);
    }
    return w.used + 256;
}

// h to particle order in FP64 (and clipped for the map); unresolved queries counted.
__global__ void k_batch_h(const float *__restrict__ hsml32, const float *__restrict__ hsml_lo,
                          const int32_t *__restrict__ order,
                          const int32_t *__restrict__ qstatus, int64_t n, double *__restrict__ hsml,
                          double *__restrict__ hmap, double hmin, int32_t *__restrict__ unresolved) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    bool bad = false;
    if (s < n) {
        const int32_t i = order[s];
        const double h = (double)hsml32[s] + (double)hsml_lo[s];
        hsml[i] = h;
        if (hmap) hmap[i] = fmax(h, hmin);
        bad = (qstatus[s] & MG_Q_UNRESOLVED) != 0;
    }
    const unsigned m = __ballot_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(unresolved, __popc(m));
}

}  // namespace mg

using namespace mg;

static bool snapshot_ok(const mg_snapshot &s, int k) {
    if (s.n < k || !s.pos || !s.hsml || s.nf < 0) return false;
    if (s.nf > 0 && (!s.fields || !s.grad)) return false;
    if (s.map && (!s.mass || s.map_res < 2 || !(s.map_size > 0))) return false;
    if (s.grid_level < 0 || s.grid_level > 9 || s.brick_threshold < 0) return false;
    return true;
}

extern "C" size_t mg_batched_workspace_bytes(const mg_snapshot *snaps, int32_t nsnap, int32_t k) {
    if (!snaps || nsnap <= 0 || k < 1 || k > MG_MAX_K) return 0;
    size_t most = 0;
    for (int i = 0; i < nsnap; ++i) {
        if (!snapshot_ok(snaps[i], k)) return 0;
        SnapPlan P;
        const size_t b = plan_snapshot(snaps[i], k, nullptr, SIZE_MAX, P);
        most = b > most ? b : most;
    }
    return most;
}

extern "C" int mg_batched_run(const mg_snapshot *snaps, int32_t nsnap, int32_t k, float radius_factor,
                              int32_t *unresolved, int64_t *stats, void *workspace, size_t workspace_bytes,
                              void *stream_) {
    if (!snaps || nsnap <= 0 || !unresolved || !workspace) return MG_ERR_ARG;
    if (k < 1 || k > MG_MAX_K) return MG_ERR_UNSUPPORTED;
    for (int i = 0; i < nsnap; ++i)
        if (!snapshot_ok(snaps[i], k)) return MG_ERR_ARG;
    if (workspace_bytes < mg_batched_workspace_bytes(snaps, nsnap, k)) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    MG_CUDA(cudaMemsetAsync(unresolved, 0, sizeof(int32_t) * nsnap, st));
    if (stats) MG_CUDA(cudaMemsetAsync(stats, 0, sizeof(int64_t) * 16 * nsnap, st));
    for (int i = 0; i < nsnap; ++i) {
        const mg_snapshot &s = snaps[i];
        SnapPlan P;
        plan_snapshot(s, k, workspace, workspace_bytes, P);
        const int64_t n = s.n;
        int rc = mg_build_cells(s.pos, &P.c, P.ws_build, P.b_build, st);
        if (rc) return rc;
        rc = mg_seed_plain(&P.c, nullptr, n, k, P.seed, st);
        if (rc) return rc;
        int64_t *st_i = stats ? stats + 16 * (int64_t)i : P.stats;
        if (!stats) MG_CUDA(cudaMemsetAsync(st_i, 0, sizeof(int64_t) * 16, st));
        rc = mg_knn_hsml(&P.c, nullptr, n, k, P.seed, radius_factor, s.level_bias, 16, P.ngb, P.hsml32, P.hsml_lo,
                         P.qstatus,
                         st_i, P.ws_knn, P.b_knn, st);
        if (rc) return rc;
        const double hmin = s.map ? 2.0 * s.map_size / (double)s.map_res : 0.0;
        k_batch_h<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(P.hsml32, P.hsml_lo, P.c.order, P.qstatus, n, s.hsml,
                                                                P.hmap,
                                                                hmin, unresolved + i);
        MG_CHECK_LAUNCH();
        if (s.nf > 0) {
            rc = mg_load_fields(&P.c, s.fields, s.nf, P.fhi, P.flo, st);
            if (rc) return rc;
            rc = mg_grad_sweep(&P.c, nullptr, n, P.ngb, k, P.hsml32, P.hsml_lo, 1, 1, P.fhi, P.flo, s.nf, P.c.order,
                               s.grad,
                               nullptr, P.gstatus, 30.0f, P.ws_grad, P.b_grad, st);
            if (rc) return rc;
        }
        if (s.map) {
            rc = mg_surface_density(s.pos, P.hmap, s.mass, n, s.map_cx, s.map_cy, s.map_size, s.map_res, 0, s.map,
                                    P.ws_sd, P.b_sd, st);
            if (rc) return rc;
        }
    }
    return MG_OK;
}
