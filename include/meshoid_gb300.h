/*
 * meshoid_gb300 -- C ABI of the GB300 (sm_103a) particle-neighbourhood path.
 *
 * Every entry point takes device pointers, plain sizes and a CUDA stream
 * (passed as void*, NULL = legacy default stream), is stream-ordered, and
 * returns an int status (MG_OK = 0).  Buffers are allocated by the caller;
 * scratch memory is passed in as a workspace whose size the matching
 * *_workspace_bytes function reports.  No entry point synchronises the stream
 * unless its comment says so.
 *
 * Particle data lives in "slot" order: the Morton order of the particles'
 * cells.  mg_build_cells computes the order and the slot/particle maps; every
 * later call indexes particles by slot.  Neighbour lists hold slots.
 *
 * Reference interfaces replaced (paths relative to the meshoid project root):
 *   mg_build_cells      cKDTree(pos, boxsize)                 src/meshoid/Meshoid.py:142-145
 *   mg_seed_plain,
 *   mg_seed_features,
 *   mg_mlp_forward      (no counterpart: first-guess radius for the search)
 *   mg_knn_hsml         tree.query(pos[mask], des_ngb) +      src/meshoid/Meshoid.py:147-170
 *                       HsmlIter(ngbdist, error_norm, dim)    src/meshoid/kernel_density.py:15-56
 *   mg_hsml_solve       HsmlIter(ngbdist, error_norm, dim)    src/meshoid/kernel_density.py:15-56
 *   mg_density          density / vol from h                  src/meshoid/Meshoid.py:169-170
 *   mg_neighbor_dist    ngbdist of tree.query                 src/meshoid/Meshoid.py:157,201-211
 *   mg_load_fields      np.take(f, ngb) operand staging       src/meshoid/Meshoid.py:258,291
 *   mg_load_fields3     the same, three FP32 planes           src/meshoid/Meshoid.py:258,291
 *   mg_hsml_polish      HsmlIter root in float-float          src/meshoid/kernel_density.py:15-56
 *   mg_grad2_moments    order-2 weights (cached moments)      src/meshoid/derivatives.py:56-138, Meshoid.py:110-140
 *   mg_grad2_solve      D order 2 / D2 contraction            src/meshoid/Meshoid.py:237-295
 *   mg_grad_sweep       gradient_weights + einsum of D / D2   src/meshoid/derivatives.py:118-138,
 *                                                             src/meshoid/Meshoid.py:237-295
 *   mg_kernel_average   get_kernel_weights + KernelAverage    src/meshoid/Meshoid.py:172-177,368-381
 *   mg_kernel_variance  KernelVariance                        src/meshoid/Meshoid.py:351-366
 *   mg_surface_density  GridSurfaceDensity(_conservative)     src/meshoid/grid_deposition.py:123-295
 *   mg_grid_density     GridDensity (DepositToGrid)           src/meshoid/grid_deposition.py:534-600,
 *                                                             src/meshoid/Meshoid.py:557-593
 *   mg_ppz_cube         Grid_PPZ_DataCube                     src/meshoid/grid_deposition.py:339-392
 *   mg_weighted_interp3d WeightedGridInterp3D                 src/meshoid/grid_deposition.py:439-531
 *   mg_radtransfer      radtransfer(_singlethread)            src/meshoid/radiation/radtransfer.py:11-200
 *   mg_kernel_weights   get_kernel_weights                    src/meshoid/Meshoid.py:172-177
 *   mg_gradient_weights gradient_weights (ComputeDWeights)    src/meshoid/derivatives.py:118-138
 *   mg_kde_1d           KDE                                   src/meshoid/Meshoid.py:722-750
 *   mg_nn_query         tree.query(target_points) (k=1)       src/meshoid/Meshoid.py:407-411
 *   (Reconstruct/Slice  f[nn] + dx.D(f) (+ D2 terms)          src/meshoid/Meshoid.py:383-502:
 *                       mg_nn_query, then mg_knn_hsml + mg_grad_sweep on the nearest-particle subset)
 *   mg_mlp_train_step   (no counterpart: trains the seed network)
 *   mg_batched_run      (no counterpart: a loop of Meshoid(...), D, SurfaceDensity over snapshots)
 */
#ifndef MESHOID_GB300_H
#define MESHOID_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MG_OK 0
#define MG_ERR_ARG 1          /* invalid argument (size, dimension, null pointer, workspace too small) */
#define MG_ERR_CUDA 2         /* a CUDA runtime call or kernel launch failed */
#define MG_ERR_NOT_CONVERGED 3 /* some queries exhausted the search-pass cap; see the per-query status */
#define MG_ERR_UNSUPPORTED 4  /* compiled limits exceeded (e.g. k > MG_MAX_K) */
#define MG_ERR_NOALLOC_LIMIT 5 /* request larger than the fixed scratch of mg_grad_sweep_noalloc */

#define MG_MAX_K 128          /* largest des_ngb the search supports */
#define MG_MAX_FIELDS 32      /* field components per gradient sweep launch */
#define MG_MLP_IN 54          /* seed network: inputs (27 cells x 2 levels) */
#define MG_MLP_IN_PAD 64      /* feature row stride (bf16 elements) */
#define MG_MLP_HIDDEN 64

/* per-query status bits written by mg_knn_hsml / mg_grad_sweep */
#define MG_Q_UNRESOLVED 1     /* search passes exhausted: neighbour set / h not final */
#define MG_Q_BAND_FP64 2      /* the k-th neighbour was re-decided with FP64 distances */
#define MG_Q_SINGULAR 4       /* moment matrix singular: pseudo-inverse used */
#define MG_Q_FP64_SOLVE 8     /* derivatives of this row re-solved in FP64 (ill-conditioned or FP32 error estimate) */
#define MG_Q_REFINED 16       /* order-2 derivatives of this row refined by one compensated FP32 step */

/* Return a static string describing a status code. */
const char *mg_status_string(int status);
/* Library version: major*10000 + minor*100 + patch. */
int mg_version(void);
/* Number of kernels this library has launched in the process so far. */
int64_t mg_launch_count(void);

/* ---- spatial index ------------------------------------------------------ */
typedef struct mg_cells {
    int64_t n;            /* particles */
    int32_t dim;          /* 1, 2 or 3 (missing coordinates are zero) */
    int32_t grid_level;   /* dense cell table level: 2^grid_level cells per side, 1..9 */
    double boxsize;       /* > 0: periodic cube [0, boxsize)^3; <= 0: open boundaries */
    /* caller-allocated device buffers, filled by mg_build_cells */
    double *frame;        /* 8: origin[3], side, 1/side, centre[3] */
    uint64_t *keys;       /* n: 63-bit Morton keys, ascending */
    int32_t *order;       /* n: slot -> particle index */
    int32_t *rank;        /* n: particle index -> slot */
    float *pos_hi;        /* 4n: float4 per slot, (x,y,z) - centre rounded to FP32, w = 0 */
    float *pos_lo;        /* 4n: float4 per slot, FP32 residual of (x,y,z) - centre - hi */
    double *pos64;        /* 3n: FP64 coordinates per slot */
    uint32_t *cell_start; /* 8^grid_level + 1: first slot of each grid cell */
    /* Optional refinement tables below the dense level ("bricks"): a cell
     * holding more than brick_threshold particles gets a table of the first
     * slots of its 8^3 descendants three levels down, recursively, so a cell
     * at any level is found in one dependent lookup per three levels instead
     * of a binary search.  brick_capacity 0 (or NULL pointers) disables them. */
    int32_t *brick_of;       /* 8^grid_level: brick index of each dense cell, -1 if none */
    uint32_t *bricks;        /* brick_capacity x MG_BRICK_WORDS */
    int32_t brick_capacity;
    int32_t brick_threshold;
} mg_cells;

#define MG_BRICK_WORDS 1028  /* 513 first slots, 512 child bricks, range begin/end, pad */
/* Bricks mg_build_cells may create for n particles (upper bound). */
int32_t mg_brick_capacity(int64_t n, int grid_level, int threshold);

/* Suggested dense-table level for n particles: the finest L with
 * 8^(L+1) <= 4n, at most 9. */
int mg_default_grid_level(int64_t n);
/* Workspace bytes mg_build_cells needs. */
size_t mg_build_cells_workspace_bytes(int64_t n, int grid_level);
/* Sort particles into Morton order and build the cell table.
 * pos: (n, dim) FP64 row-major device array in particle order.  Replaces
 * cKDTree construction (src/meshoid/Meshoid.py:142-145). */
int mg_build_cells(const double *pos, mg_cells *cells, void *workspace, size_t workspace_bytes,
                   void *stream);

/* ---- seeds (first-guess smoothing lengths) ------------------------------ */
/* Plain seed: h from the particle count of the query's own adaptive cell.
 * queries: nq slots (NULL = all n slots in order).  seed_h: nq FP32. */
int mg_seed_plain(const mg_cells *cells, const int32_t *queries, int64_t nq, int32_t k,
                  float *seed_h, void *stream);
/* Seed-network inputs: log2(1 + count) of the 27 cells around the query at the
 * level below its adaptive level and at the adaptive level itself (the finest
 * level whose cell holds >= max(2, k/4) particles): 54 values, bf16, row
 * stride MG_MLP_IN_PAD, padding zero; plus the adaptive cell side (FP32). */
int mg_seed_features(const mg_cells *cells, const int32_t *queries, int64_t nq, int32_t k,
                     uint16_t *features, float *cell_side, void *stream);
/* Seed network forward: 54 -> 64 -> 64 -> 1, GELU, bf16 weights, FP32
 * accumulation (tensor cores).  Weights: w1 (64 x 64, input-padded, bf16),
 * b1 (64 FP32), w2 (64 x 64 bf16), b2 (64), w3 (64 bf16), b3 (1).  out:
 * log(h / cell_side) per row (FP32).  If seed_h is non-NULL it also receives
 * exp(out) * cell_side. */
int mg_mlp_forward(const uint16_t *features, int64_t n, const uint16_t *w1, const float *b1,
                   const uint16_t *w2, const float *b2, const uint16_t *w3, const float *b3,
                   const float *cell_side, float *out, float *seed_h, void *stream);
/* One Adam step of the seed network on a batch (mean squared error on
 * log(h / cell_side)).  params: FP32 master copy of all weights (layout in
 * MG_MLP_PARAM_COUNT order: w1, b1, w2, b2, w3, b3), adam_m / adam_v same
 * size, bf16 copies (w1, w2, w3) refreshed after the step.  target: n FP32.
 * loss_out: device FP32 scalar (mean loss of the batch before the step).
 * grads_out (optional, may be NULL): FP32 gradient of the loss w.r.t. params. */
#define MG_MLP_PARAM_COUNT (64 * 64 + 64 + 64 * 64 + 64 + 64 + 1)
int mg_mlp_train_step(const uint16_t *features, const float *target, int64_t n, float *params,
                      float *adam_m, float *adam_v, int32_t step, float lr, uint16_t *w1_bf16,
                      uint16_t *w2_bf16, uint16_t *w3_bf16, float *loss_out, float *grads_out,
                      void *workspace, size_t workspace_bytes, void *stream);
size_t mg_mlp_train_workspace_bytes(int64_t n);

/* ---- neighbours + smoothing lengths ------------------------------------- */
/* Workspace bytes for mg_knn_hsml with nq queries of k neighbours. */
size_t mg_knn_hsml_workspace_bytes(int64_t nq, int32_t k);
/* k nearest neighbours (self included) of each query and its smoothing length
 * h solving norm * sum_j W(d_j / h) = k over those neighbours.
 *   seed_h: nq FP32 first guesses of h; the first search radius is
 *           radius_factor * seed_h.  A query whose radius holds fewer than k
 *           particles (or too many) is re-queued with a corrected radius, up to
 *           max_passes passes.
 *   level_bias: 0 or 1 -- the searched cells have side >= R / 2^level_bias
 *           (finer cells: fewer candidates, more cell lookups).
 *   ngb:    nq * k slots, unordered within a row (the set is exact: the k
 *           smallest by (FP64 d^2, particle index)).
 *   hsml:   nq FP32.  hsml_lo: NULL, or nq FP32 -- then h = hsml + hsml_lo:
 *           for k <= 32 the float-float root (distances and the last Newton
 *           step in float-float, ~1e-12 relative); for k > 32 the FP32
 *           solve's last step kept as an unevaluated sum (~1e-8; polish it
 *           with mg_hsml_polish).  hsml alone is good to ~1e-7.
 *           qstatus: nq MG_Q_* bits.
 *   stats:  16 int64 device counters, accumulated (the caller zeroes them):
 *           [0] passes after the first, [1] candidates scanned (warp passes)
 *           or staged (first pass, per query it serves), [2] retries,
 *           [3] FP64 band re-decisions, [4] unresolved, [5] Newton steps,
 *           [6..8] retries for too few / too many / band outside the radius,
 *           [9] queries handed to the block-wide path (scan list > 2048).
 * Replaces tree.query + HsmlIter (src/meshoid/Meshoid.py:157,165;
 * src/meshoid/kernel_density.py:15-56). */
int mg_knn_hsml(const mg_cells *cells, const int32_t *queries, int64_t nq, int32_t k,
                const float *seed_h, float radius_factor, int32_t level_bias, int32_t max_passes,
                int32_t *ngb,
                float *hsml, float *hsml_lo, int32_t *qstatus, int64_t *stats, void *workspace,
                size_t workspace_bytes, void *stream);
/* First pass of mg_knn_hsml: 1 (default) runs it one thread per query over
 * candidates staged once per block of 128 consecutive queries, the queries it
 * cannot decide exactly going on to the warp-per-query passes; 0 runs every
 * pass warp per query.  Both give the same neighbour sets and distances.
 * Process-wide; returns the previous setting. */
int mg_knn_set_group_pass(int32_t enabled);
/* Passes after the first of mg_knn_hsml: 1 runs them in one cooperative
 * launch that drains the device-side work queue (the warp path, a grid-wide
 * barrier, the block-wide path for crowded queries, a barrier; it ends when a
 * pass starts on an empty queue); 0 (the default) launches the kernels of
 * every pass from the host (max_passes of them, most on an empty queue).
 * Both give the same neighbour sets, distances and h; measured on a GB300
 * the cooperative launch is no faster on one snapshot (as fast on a Plummer
 * sphere, 3% slower on a clump mixture) and keeps concurrent streams from
 * overlapping.  Process-wide; returns the previous setting. */
int mg_knn_set_persistent_passes(int32_t enabled);
/* Smoothing lengths, densities and volumes in output-row order
 * (src/meshoid/Meshoid.py:169-170): for query q, row r = out_rows[q] (or q),
 * h_out[r] = hsml[q] + hsml_lo[q] (FP64; hsml_lo may be NULL),
 * density[r] = des_ngb m_rows[r] / (volnorm h^dim),
 * vol[r] = m_rows[r] / density[r]; volnorm = 2, pi, 4 pi / 3.  m_rows NULL
 * means unit masses; density / vol may be NULL. */
int mg_density(const int32_t *out_rows, const float *hsml, const float *hsml_lo, int64_t nq, const double *m_rows,
               int32_t des_ngb, int32_t dim, double *h_out, double *density, double *vol, void *stream);
/* Smoothing lengths from given neighbour distances (HsmlIter,
 * src/meshoid/kernel_density.py:15-56, without a neighbour search): d2 holds
 * nq rows of k squared distances (FP32, any order, self included as 0);
 * hsml (nq FP32) solves norm * sum_j W(d_j / h) = k by bracketed Newton to
 * ~2e-7 relative.  stats (optional): stats[5] += Newton steps. */
int mg_hsml_solve(const float *d2, int64_t nq, int32_t k, int32_t dim, float *hsml, int64_t *stats, void *stream);
/* FP64 distances of each row of ngb, sorted ascending with the row's slots
 * (ties by particle index).  Outputs particle indices (int64) and distances in
 * the layout of cKDTree.query (src/meshoid/Meshoid.py:157). */
int mg_neighbor_dist(const mg_cells *cells, const int32_t *queries, int64_t nq, const int32_t *ngb,
                     int32_t k, int64_t *ngb_particles, double *dist, void *stream);

/* ---- fields and derivatives --------------------------------------------- */
/* Gather f (n, nf) FP64 particle order into slot order as an FP32 pair
 * hi + lo = f (to ~48 bits).  Both outputs are (n, nfp) row-major with
 * nfp = nf rounded up to a multiple of 4 (padding zero); lo may be NULL. */
int mg_load_fields(const mg_cells *cells, const double *f, int32_t nf, float *hi, float *lo,
                   void *stream);
/* Kernel-weighted least-squares derivatives of nf field components in one
 * neighbour sweep (src/meshoid/derivatives.py:27-138, src/meshoid/Meshoid.py:
 * 237-295).  order 1: first derivatives (dim per component) into d1;
 * order 2: first derivatives of the second-order fit into d1 and the
 * dim*(dim+1)/2 second derivatives ([xx,yy,zz,xy,yz,zx] in 3-D) into d2.
 * Outputs are FP32, row-major by output row r = out_rows[q] (r = q when
 * out_rows is NULL): d1[(r * nf + c) * dim + a], d2[(r * nf + c) * nd2 + m].  f_lo may be NULL (fields exactly representable
 * in FP32).  hsml_lo (may be NULL): low parts of h (mg_knn_hsml), used for
 * the 1/h scaling of the separations.  qstatus (optional) gets MG_Q_SINGULAR
 * bits.
 * The sweep runs in FP32 (normal equations scaled by 1/h, Cholesky).  With a
 * workspace (mg_grad_sweep_workspace_bytes), rows whose moment matrix has an
 * estimated condition number above cond_threshold, or is singular, are
 * re-solved in FP64 from the FP64 positions (pseudo-inverse when singular).
 * workspace NULL disables the re-solve. */
size_t mg_grad_sweep_workspace_bytes(int64_t nq);
/* Order-2 refinement step of mg_grad_sweep (and mg_grad_sweep_noalloc),
 * process-wide, off by default (not in the reference).  On: a row whose FP32
 * answer may miss the tolerance of its second-derivative part through the
 * matrix rounding (~6e-8 cond ||x||) is refined once in FP32, with the
 * residual f_j - f_i - a_j . x carried in float-float, and marked
 * MG_Q_REFINED, instead of going to the FP64 re-solve; singular rows and rows
 * with a condition estimate above cond_threshold still do.  Returns the
 * previous setting. */
int mg_grad_set_refine(int32_t enabled);
int mg_grad_sweep(const mg_cells *cells, const int32_t *queries, int64_t nq, const int32_t *ngb,
                  int32_t k, const float *hsml, const float *hsml_lo, int32_t order, int32_t weighted, const float *f_hi,
                  const float *f_lo, int32_t nf, const int32_t *out_rows, float *d1, float *d2,
                  int32_t *qstatus, float cond_threshold, void *workspace, size_t workspace_bytes,
                  void *stream);
/* mg_grad_sweep for callers that cannot allocate device memory (a host code
 * that has reserved its whole GPU memory budget for its own pool, or a loop
 * whose owner forbids allocator calls).  No counterpart in the reference.
 * Same arguments and results as mg_grad_sweep, minus the workspace: the
 * FP64 re-solve queue and its row marks live in a fixed array inside this
 * library (about 16 MiB, resident on each GPU that loads the library until the
 * process exits).
 * Rejects nq > MG_NOALLOC_MAX_QUERIES with MG_ERR_NOALLOC_LIMIT.  All calls
 * share that array: calls that overlap on the GPU race.  A call's results
 * depend on the array until its last kernel has finished on the GPU, so the
 * caller orders whole calls on the GPU (one stream, or a wait on an event
 * recorded after the previous call), not only on the host.  The queue counter
 * is cleared at the start of every call.  Each call looks up the array's
 * address on the current device (no cached address survives a device reset);
 * a device's first call also loads the library's module there, so make it
 * before any stream capture. */
#define MG_NOALLOC_MAX_QUERIES (1 << 21)
int mg_grad_sweep_noalloc(const mg_cells *cells, const int32_t *queries, int64_t nq, const int32_t *ngb,
                          int32_t k, const float *hsml, const float *hsml_lo, int32_t order, int32_t weighted, const float *f_hi,
                          const float *f_lo, int32_t nf, const int32_t *out_rows, float *d1, float *d2,
                          int32_t *qstatus, float cond_threshold, void *stream);
/* ---- order-2 derivatives in float-float --------------------------------- */
/* The order-2 fit (D order 2, D2: src/meshoid/derivatives.py:27-138,
 * src/meshoid/Meshoid.py:110-140, 237-295) is sensitive at 32 neighbours:
 * FP32 rounding of the separations alone moves the FP64 answer by more than
 * 1e-5 on many rows.  These entry points carry separations, weights, basis,
 * moment matrix and right-hand sides as float-float pairs and solve by
 * iterative refinement; rows that are singular or ill-conditioned in FP32
 * use the FP64 inverse (pseudo-inverse when singular) of the float-float
 * moment matrix.
 *
 * mg_hsml_polish: the root of HsmlIter's equation (kernel_density.py:15-56)
 * to float-float precision, hsml_hi + hsml_lo, from the FP32 smoothing
 * lengths hsml of mg_knn_hsml and the neighbour rows (two Newton steps with
 * the neighbour count in float-float).  hsml_hi may alias hsml. */
int mg_hsml_polish(const mg_cells *cells, const int32_t *queries, int64_t nq, const int32_t *ngb, int32_t k,
                   const float *hsml, float *hsml_hi, float *hsml_lo, void *stream);
/* Gather f (n, nf) FP64 particle order into slot order as three FP32 planes
 * hi + mid + lo = f (to ~2^-72 of |f|), each (n, nfp) row-major, nfp = nf
 * rounded up to a multiple of 4.  Differences of neighbours whose values
 * agree to many digits keep their precision (two planes keep 2^-48 of |f|). */
int mg_load_fields3(const mg_cells *cells, const double *f, int32_t nf, float *hi, float *mid, float *lo,
                    void *stream);
/* Per-row float-float Cholesky factors of the order-2 moment matrices (the
 * analogue of the reference's cached dweights_3rdorder / d2weights,
 * Meshoid.py:110-140), into a caller buffer of mg_grad2_moments_bytes(nq,
 * dim) bytes that mg_grad2_solve reads.  hsml_lo may be NULL.  Rows whose
 * matrix is not positive definite, or whose condition estimate exceeds
 * cond_threshold, are queued in the same buffer for the FP64 re-solve of
 * every mg_grad2_solve call (FP64 positions and fields, the reference's
 * arithmetic). */
size_t mg_grad2_moments_bytes(int64_t nq, int32_t dim);
int mg_grad2_moments(const mg_cells *cells, const int32_t *queries, int64_t nq, const int32_t *ngb, int32_t k,
                     const float *hsml, const float *hsml_lo, int32_t weighted, float cond_threshold,
                     void *moments, size_t moments_bytes, void *stream);
/* Order-2 derivatives of nf components (three-plane fields of
 * mg_load_fields3) from the moments of the same rows, h and weighting
 * (float-float right-hand sides solved with the cached factors):
 * d1[(r * nf + c) * dim + a] first derivatives, d2 (may be NULL)
 * [(r * nf + c) * nd2 + m] second derivatives, r = out_rows[q] (q when NULL),
 * FP32.  qstatus (optional): MG_Q_FP64_SOLVE on rows solved with the FP64
 * inverse, MG_Q_SINGULAR when that is a pseudo-inverse.  workspace:
 * mg_grad2_solve_workspace_bytes(nq) bytes. */
size_t mg_grad2_solve_workspace_bytes(int64_t nq);
int mg_grad2_solve(const mg_cells *cells, const int32_t *queries, int64_t nq, const int32_t *ngb, int32_t k,
                   const float *hsml, const float *hsml_lo, int32_t weighted, void *moments, size_t moments_bytes,
                   const float *f_hi, const float *f_mid, const float *f_lo, int32_t nf, const int32_t *out_rows,
                   float *d1, float *d2, int32_t *qstatus, void *workspace, size_t workspace_bytes, void *stream);
/* Kernel-weighted neighbour average K(d/h)/sum K . f[ngb] of nf components
 * (src/meshoid/Meshoid.py:172-177,368-381).  out: (rows, nf) FP64, row
 * out_rows[q] (or q). */
int mg_kernel_average(const mg_cells *cells, const int32_t *queries, int64_t nq, const int32_t *ngb,
                      int32_t k, const float *hsml, const float *f_hi, const float *f_lo, int32_t nf,
                      const int32_t *out_rows, double *out, void *stream);

/* Population standard deviation of nf components over each query's k
 * neighbours, self included (np.std(f[ngb], axis=1) of
 * src/meshoid/Meshoid.py:351-366).  out: (rows, nf) FP64, row out_rows[q] (or q). */
int mg_kernel_variance(const mg_cells *cells, const int32_t *queries, int64_t nq, const int32_t *ngb, int32_t k,
                       const float *f_hi, const float *f_lo, int32_t nf, const int32_t *out_rows, double *out,
                       void *stream);

/* ---- maps ---------------------------------------------------------------- */
size_t mg_surface_density_workspace_bytes(int64_t n, int32_t res);
/* Column-integrated cubic-spline deposition onto a res x res grid of
 * sightlines (src/meshoid/grid_deposition.py:123-295).  pos (n,3) FP64,
 * h and f (n) FP64, all particle order.  grid (res*res) FP64, indexed
 * [gx * res + gy], pixel nodes at g * size / (res - 1) from the corner
 * (cx - size/2, cy - size/2).  conservative != 0 selects the per-particle
 * normalised deposit of GridSurfaceDensity_conservative_core. */
int mg_surface_density(const double *pos, const double *h, const double *f, int64_t n, double cx,
                       double cy, double size, int32_t res, int32_t conservative, double *grid,
                       void *workspace, size_t workspace_bytes, void *stream);
/* 3-D deposition (src/meshoid/grid_deposition.py), positions n x 3 FP64 in
 * any order, grids C-order FP64 [gx][gy][gz] on the device, written in full.
 * FP32 kernel weights on FP64 node ranges (the reference's truncation and
 * clipping / wrap); FP64 atomic deposits.
 * GridDensity (:534-600, DepositToGrid Meshoid.py:557-593): nodes g * dx
 * (dx = size / (res - 1)) from the corner centre - size/2 + dx/2; each
 * particle's f spread by its kernel weights normalised to 1; grid / dx^3.
 * periodic != 0: ranges are not clipped and wrap modulo res (box_size >= 0);
 * a particle whose cube then spans more than 4 res + 8 nodes on an axis is
 * not deposited and counted in n_skipped (optional device int64).
 * Non-wrapping cubes are accumulated per 8^3-node tile in shared memory:
 * mg_grid_density_count writes a bound of their (tile, particle) overlaps to
 * *npairs (device int64), which the caller reads to size the workspace and
 * passes on. */
int mg_grid_density_count(const double *pos, const double *h, int64_t n, double cx, double cy, double cz,
                          double size, int32_t res, int32_t periodic, int64_t *npairs, void *stream);
size_t mg_grid_density_workspace_bytes(int64_t n, int64_t npairs, int32_t res);
int mg_grid_density(const double *pos, const double *h, const double *f, int64_t n, double cx, double cy,
                    double cz, double size, int32_t res, int32_t periodic, double *grid, int64_t *n_skipped,
                    int64_t npairs, void *workspace, size_t workspace_bytes, void *stream);
/* Grid_PPZ_DataCube (:339-392): res_xy x res_xy x res_z cube; plane nodes
 * g * size_xy / (res_xy - 1), data nodes g * size_z / (res_z - 1) from
 * (cx, cy, cz) - sizes / 2; z, hz: the data coordinate and its width. */
int mg_ppz_cube(const double *pos, const double *h, const double *f, const double *z, const double *hz, int64_t n,
                double cx, double cy, double cz, double size_xy, double size_z, int32_t res_xy, int32_t res_z,
                double *grid, void *stream);
/* WeightedGridInterp3D (:439-531): cell-centre nodes; result = sum f wt W /
 * sum wt W with per-particle normalised W; weight (res^3 scratch) receives the
 * denominator.  Cells no particle reaches are NaN and counted in n_empty
 * (optional device int64): the reference gives them the nearest particle's
 * f, which the caller fills (mg_nn_query). */
int mg_weighted_interp3d(const double *pos, const double *h, const double *f, const double *wt, int64_t n,
                         double cx, double cy, double cz, double size, int32_t res, double *result, double *weight,
                         int64_t *n_empty, void *stream);
/* Emission/absorption ray tracing along z (radtransfer_singlethread,
 * src/meshoid/radiation/radtransfer.py:87-200): for each pixel node g * dx
 * (dx = L / (res - 1)) from (cx, cy) - L/2, the particles whose footprint
 * (h at least dx) holds it, from the largest z - cz to the smallest (ties by
 * index): I <- exp(-tau) I - expm1(-tau) j / (4 pi kappa + 1e-100), tau =
 * kappa kernel2d(r/h) m / h^2.  j, kappa: n x bands (bands <= 8); i0: bands
 * background intensities or NULL; intensity, tau (optional): res x res x
 * bands FP64.  FP32 per-pixel walk on FP64 footprints.
 * mg_radtransfer_count writes the number of (32 x 32-pixel tile, particle)
 * overlaps to *npairs (device int64); the caller reads it to size the
 * workspace (mg_radtransfer_workspace_bytes) and passes it on. */
int mg_radtransfer_count(const double *pos, const double *h, const double *m, int64_t n, int32_t res, double L,
                         double cx, double cy, int64_t *npairs, void *stream);
size_t mg_radtransfer_workspace_bytes(int64_t n, int64_t npairs, int32_t res, int32_t bands);
int mg_radtransfer(const double *j, const double *m, const double *kappa, const double *pos, const double *h,
                   int64_t n, int32_t bands, int32_t res, double L, double cx, double cy, double cz,
                   const double *i0, int64_t npairs, double *intensity, double *tau, void *workspace,
                   size_t workspace_bytes, void *stream);
/* Explicit weights (FP64) for callers that read them; the derivative and
 * average entry points never need them.
 * mg_kernel_weights: w[q][j] = Kernel(d[q][j] / h[q]) / sum_j Kernel(...)
 * (get_kernel_weights, src/meshoid/Meshoid.py:172-177); ngbdist nq x k.
 * mg_gradient_weights: (nq, nd, k) least-squares derivative weights of
 * src/meshoid/derivatives.py:27-138 (nd = dim at order 1; 2/5/9 at order 2
 * in 1/2/3-D), pos N x dim, ngb nq x k particle indices, indices nq query
 * particles, boxsize <= 0: no box.  An exactly singular normal matrix (the
 * reference raises LinAlgError) leaves its row NaN and is counted in
 * n_singular (optional device int64).
 * mg_kde_1d: f[g] = sum over particles with |grid[g] - x| <= bw of
 * Kernel(|grid[g] - x| / bw) / bw * 4/3 (KDE, src/meshoid/Meshoid.py:722-750). */
int mg_kernel_weights(const double *ngbdist, const double *h, int64_t nq, int32_t k, double *w, void *stream);
int mg_gradient_weights(const double *pos, int32_t dim, const int64_t *ngb, int32_t k, const double *h,
                        const int64_t *indices, int64_t nq, double boxsize, int32_t weighted, int32_t order,
                        double *out, int64_t *n_singular, void *stream);
size_t mg_kde_1d_workspace_bytes(int64_t ng);
int mg_kde_1d(const double *x, const double *bw, int64_t n, const double *grid, int64_t ng, double *f,
              void *workspace, size_t workspace_bytes, void *stream);
/* Nearest particle of each target point (k = 1 query of
 * src/meshoid/Meshoid.py:410): nn (nt) particle indices, ties by index. */
size_t mg_nn_query_workspace_bytes(int64_t nt);
int mg_nn_query(const mg_cells *cells, const double *targets, int64_t nt, int64_t *nn,
                void *workspace, size_t workspace_bytes, void *stream);

/* ---- many snapshots in one stream-ordered call ----------------------------
 * No counterpart in the reference (its caller loops over snapshots, one
 * Meshoid each).  For each snapshot, in order: cell index, plain seed,
 * neighbours + h (des_ngb = k), first derivatives of its nf field components
 * (order 1, weighted) and, if map != NULL, the column density of its masses
 * on a map_res^2 grid with h clipped below at 2 map_size / map_res (the
 * defaults of Meshoid.SurfaceDensity, src/meshoid/Meshoid.py:595-643).  No
 * host synchronisation and no allocation inside: the call can be captured in
 * one CUDA graph and replayed.  Scratch is reused from one snapshot to the
 * next (stream order), so the workspace is the largest snapshot's need. */
typedef struct mg_snapshot {
    int64_t n;               /* particles */
    const double *pos;       /* n x 3 FP64 */
    const double *mass;      /* n FP64, deposited on the map (NULL when map == NULL) */
    const double *fields;    /* n x nf FP64 row-major (NULL when nf == 0) */
    int32_t nf;              /* field components */
    int32_t grid_level;      /* dense cell-table level (0: mg_default_grid_level(n)) */
    int32_t level_bias;      /* 0 or 1 (mg_knn_hsml) */
    int32_t brick_threshold; /* refinement tables for cells above this count (0: none) */
    double *hsml;            /* out: n FP64 smoothing lengths, particle order */
    float *grad;             /* out: n x nf x 3 FP32 first derivatives, particle order */
    double *map;             /* out: map_res x map_res FP64 (NULL: no map) */
    double map_cx, map_cy, map_size;
    int32_t map_res;
    int32_t reserved;
} mg_snapshot;
size_t mg_batched_workspace_bytes(const mg_snapshot *snaps, int32_t nsnap, int32_t k);
/* snaps: host array of nsnap descriptors (device pointers inside).
 * unresolved: nsnap int32 device counters (zeroed here), the number of
 * queries whose search did not finish within 16 passes (0 normally).
 * stats (optional): nsnap x 16 int64 device counters of mg_knn_hsml. */
int mg_batched_run(const mg_snapshot *snaps, int32_t nsnap, int32_t k, float radius_factor,
                   int32_t *unresolved, int64_t *stats, void *workspace, size_t workspace_bytes,
                   void *stream);

#ifdef __cplusplus
}
#endif
#endif /* MESHOID_GB300_H */
