/*
 * CPU oracle for the meshoid particle-neighbourhood path (TEST INFRASTRUCTURE).
 *
 * A plain-C, FP64 restatement of the reference algorithms, used only by the
 * test-suite, by __graft_entry__.smoke() and by bench.py's CPU-baseline arm as
 * the checker / the timed CPU path. Nothing in the product (meshoid_gb300/)
 * links or calls this file.
 *
 * Each function cites the reference source it follows (paths relative to the
 * meshoid project root, version 1.46.0).  The reference runs these loops as
 * Numba @njit(fastmath=True) host code; here they are compiled as strict IEEE
 * FP64 (no contraction) so the oracle is reproducible across x86 and Arm.
 * Outer loops over particles are OpenMP-parallel, as the reference's prange.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* src/meshoid/kernel_density.py:82-96 (Kernel): un-normalised cubic spline. */
static inline double spline_w(double q) {
    if (q <= 0.5) return 1.0 - 6.0 * q * q + 6.0 * q * q * q;
    if (q <= 1.0) {
        double a = 1.0 - q;
        return 2.0 * a * a * a;
    }
    return 0.0;
}

/* src/meshoid/kernel_density.py:61-68 (kernel2d): 2-D normalised spline, q <= 1. */
static inline double spline_2d(double q) {
    double k;
    if (q <= 0.5) {
        k = 1.0 - 6.0 * q * q * (1.0 - q);
    } else {
        double a = 1.0 - q;
        k = 2.0 * a * a * a;
    }
    return k * 1.8189136353359467;
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/*
 * src/meshoid/kernel_density.py:15-56 (HsmlIter).  Bisection on the kernel-
 * weighted neighbour count n(h) = norm * sum_j W(d_j / h) until
 * |n - des_ngb| <= error_norm; the output is the last midpoint.  The reference
 * has no iteration cap; `max_iter` bounds the loop here and the number of
 * particles that hit it is returned.
 */
int64_t orc_hsml_iter(const double *ngbdist, int64_t n, int k, int dim,
                      double error_norm, int max_iter, double *hsml) {
    double norm = (dim == 3) ? 32.0 / 3.0 : (dim == 2 ? 40.0 / 7.0 : 8.0 / 3.0);
    double bound_coeff = 1.0 / (1.0 - pow(2.0 * norm, -1.0 / 3.0));
    int64_t capped = 0;
#pragma omp parallel for schedule(static) reduction(+ : capped)
    for (int64_t i = 0; i < n; ++i) {
        const double *d = ngbdist + i * k;
        double upper = d[k - 1] * bound_coeff;
        double lower = d[1];
        double err = 1e100, h = 0.0;
        int it = 0;
        while (err > error_norm) {
            h = (upper + lower) * 0.5;
            double nn = 0.0;
            for (int j = 0; j < k; ++j) {
                double q = d[j] / h;
                if (q <= 0.5)
                    nn += 1.0 - 6.0 * q * q + 6.0 * q * q * q;
                else if (q <= 1.0) {
                    double a = 1.0 - q;
                    nn += 2.0 * a * a * a;
                }
            }
            nn *= norm;
            if (nn > (double)k)
                upper = h;
            else
                lower = h;
            err = fabs(nn - (double)k);
            if (++it >= max_iter) {
                capped += 1;
                break;
            }
        }
        hsml[i] = h;
    }
    return capped;
}

/* src/meshoid/derivatives.py:9-15 (nearest_image). */
static inline double nearest_image(double dx, double box) {
    if (fabs(dx) > box * 0.5) return -copysign(box - fabs(dx), dx);
    return dx;
}

/* Gauss-Jordan inverse with partial pivoting (stands in for np.linalg.inv,
 * src/meshoid/derivatives.py:132).  Returns 0 on success, 1 if singular. */
static int invert(int n, double *a, double *inv) {
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) inv[r * n + c] = (r == c) ? 1.0 : 0.0;
    for (int c = 0; c < n; ++c) {
        int p = c;
        double best = fabs(a[c * n + c]);
        for (int r = c + 1; r < n; ++r)
            if (fabs(a[r * n + c]) > best) { best = fabs(a[r * n + c]); p = r; }
        if (best == 0.0) return 1;
        if (p != c)
            for (int j = 0; j < n; ++j) {
                double t = a[c * n + j]; a[c * n + j] = a[p * n + j]; a[p * n + j] = t;
                t = inv[c * n + j]; inv[c * n + j] = inv[p * n + j]; inv[p * n + j] = t;
            }
        double piv = a[c * n + c];
        for (int j = 0; j < n; ++j) { a[c * n + j] /= piv; inv[c * n + j] /= piv; }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            double f = a[r * n + c];
            if (f == 0.0) continue;
            for (int j = 0; j < n; ++j) {
                a[r * n + j] -= f * a[c * n + j];
                inv[r * n + j] -= f * inv[c * n + j];
            }
        }
    }
    return 0;
}

/* src/meshoid/derivatives.py:107-114 (get_num_derivs). */
static int num_derivs(int dim, int order) {
    if (order == 1) return dim;
    return dim == 1 ? 2 : (dim == 2 ? 5 : 9);
}

/*
 * src/meshoid/derivatives.py:118-138 (gradient_weights) with its helpers
 * kernel_dx_and_weights :27-52 and polyfit_leastsq_matrices :56-103.
 * pos (N, dim) row-major, ngb (Nq, k) int64, h (Nq,), indices (Nq,) int64.
 * out (Nq, nd, k).  boxsize <= 0 means non-periodic.  Returns the number of
 * singular moment matrices (their rows are left zero).
 */
int64_t orc_gradient_weights(const double *pos, int dim, const int64_t *ngb, int k,
                             const double *h, const int64_t *indices, int64_t nq,
                             double boxsize, int weighted, int order, double *out) {
    int nd = num_derivs(dim, order);
    int64_t singular = 0;
#pragma omp parallel reduction(+ : singular)
    {
        double *dx = (double *)malloc(sizeof(double) * k * 3);
        double *w = (double *)malloc(sizeof(double) * k);
        double *rhs = (double *)malloc(sizeof(double) * 9 * k);
        double lhs[81], inv[81];
#pragma omp for schedule(static)
        for (int64_t i = 0; i < nq; ++i) {
            int64_t idx = indices[i];
            const int64_t *nb = ngb + i * k;
            for (int j = 0; j < k; ++j) {
                double r = 0.0;
                int64_t nj = nb[j];
                for (int c = 0; c < dim; ++c) {
                    double d = pos[nj * dim + c] - pos[idx * dim + c];
                    if (boxsize > 0) d = nearest_image(d, boxsize);
                    dx[j * 3 + c] = d;
                    r += d * d;
                }
                w[j] = weighted ? spline_w(sqrt(r) / h[i]) : 1.0;
            }
            memset(lhs, 0, sizeof(lhs));
            if (order == 1) {
                for (int j = 0; j < k; ++j)
                    for (int a = 0; a < dim; ++a) rhs[a * k + j] = w[j] * dx[j * 3 + a];
                for (int j = 0; j < k; ++j)
                    for (int a = 0; a < dim; ++a)
                        for (int b = 0; b < dim; ++b) lhs[a * nd + b] += rhs[a * k + j] * dx[j * 3 + b];
            } else {
                for (int j = 0; j < k; ++j)
                    for (int a = 0; a < nd; ++a) {
                        double v;
                        if (a < dim) v = dx[j * 3 + a];
                        else if (a < 2 * dim) { int d = a - dim; v = 0.5 * dx[j * 3 + d] * dx[j * 3 + d]; }
                        else { int d = a - 2 * dim; v = dx[j * 3 + d % dim] * dx[j * 3 + (d + 1) % dim]; }
                        rhs[a * k + j] = v;
                    }
                for (int j = 0; j < k; ++j)
                    for (int a = 0; a < nd; ++a)
                        for (int b = 0; b < nd; ++b) lhs[a * nd + b] += rhs[a * k + j] * rhs[b * k + j] * w[j];
                for (int j = 0; j < k; ++j)
                    for (int a = 0; a < nd; ++a) rhs[a * k + j] *= w[j];
            }
            double *res = out + i * nd * k;
            memset(res, 0, sizeof(double) * nd * k);
            if (invert(nd, lhs, inv)) { singular += 1; continue; }
            for (int a = 0; a < nd; ++a)
                for (int b = 0; b < nd; ++b) {
                    double c = inv[a * nd + b];
                    for (int j = 0; j < k; ++j) res[a * k + j] += c * rhs[b * k + j];
                }
        }
        free(dx); free(w); free(rhs);
    }
    return singular;
}

/*
 * src/meshoid/Meshoid.py:258,268 (D / D2 application):
 *   out[i, c, d] = sum_j W[i, row0 + d, j] * (f[ngb[i, j], c] - f[indices[i], c])
 * f (N, nc) row-major, W (Nq, nd_total, k), out (Nq, nc, nrows).
 */
void orc_apply_weights(const double *W, int nd_total, int row0, int nrows,
                       const int64_t *ngb, int k, const int64_t *indices, int64_t nq,
                       const double *f, int nc, double *out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nq; ++i) {
        const double *wi = W + i * nd_total * k;
        const int64_t *nb = ngb + i * k;
        int64_t self = indices[i];
        for (int c = 0; c < nc; ++c) {
            double f0 = f[self * nc + c];
            for (int d = 0; d < nrows; ++d) {
                const double *wr = wi + (row0 + d) * k;
                double s = 0.0;
                for (int j = 0; j < k; ++j) s += wr[j] * (f[nb[j] * nc + c] - f0);
                out[(i * nc + c) * nrows + d] = s;
            }
        }
    }
}

/* src/meshoid/Meshoid.py:172-177, 368-381 (get_kernel_weights + KernelAverage). */
void orc_kernel_average(const double *ngbdist, const int64_t *ngb, int k, const double *h,
                        int64_t nq, const double *f, double *out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nq; ++i) {
        double ksum = 0.0, acc = 0.0;
        for (int j = 0; j < k; ++j) ksum += spline_w(ngbdist[i * k + j] / h[i]);
        for (int j = 0; j < k; ++j)
            acc += spline_w(ngbdist[i * k + j] / h[i]) / ksum * f[ngb[i * k + j]];
        out[i] = acc;
    }
}

/*
 * src/meshoid/grid_deposition.py:187-229 (GridSurfaceDensity_core) and
 * :232-295 (GridSurfaceDensity_conservative_core).  Pixel nodes sit at g*dx,
 * dx = size/(res-1); grid indexed [gx, gy]; no periodic wrap.  The reference
 * gives each thread a private grid and sums them (:151-179); here each thread
 * also owns a private grid, summed at the end.
 */
void orc_surface_density(const double *f, const double *x, const double *h, int64_t n,
                         double cx, double cy, double size, int res, int conservative,
                         double *grid) {
    double dx = size / (double)(res - 1);
    int nt = orc_num_threads();
    size_t cells = (size_t)res * (size_t)res;
    double *priv = (double *)calloc((size_t)nt * cells, sizeof(double));
#pragma omp parallel
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        double *g = priv + (size_t)t * cells;
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            double xs0 = x[i * 3 + 0] - cx + size * 0.5;
            double xs1 = x[i * 3 + 1] - cy + size * 0.5;
            double hs = h[i];
            if (conservative && hs < dx) hs = dx;
            double hinv = 1.0 / hs;
            int gxmin = (int)((xs0 - hs) / dx + 1.0); if (gxmin < 0) gxmin = 0;
            int gxmax = (int)((xs0 + hs) / dx); if (gxmax > res - 1) gxmax = res - 1;
            int gymin = (int)((xs1 - hs) / dx + 1.0); if (gymin < 0) gymin = 0;
            int gymax = (int)((xs1 + hs) / dx); if (gymax > res - 1) gymax = res - 1;
            if (!conservative) {
                double mh2 = f[i] * hinv * hinv;
                for (int gx = gxmin; gx <= gxmax; ++gx) {
                    double ddx = xs0 - gx * dx; ddx *= ddx;
                    for (int gy = gymin; gy <= gymax; ++gy) {
                        double ddy = xs1 - gy * dx; ddy *= ddy;
                        double r = sqrt(ddx + ddy);
                        if (r > hs) continue;
                        g[(size_t)gx * res + gy] += spline_2d(r * hinv) * mh2;
                    }
                }
            } else {
                double tot = 0.0;
                for (int gx = gxmin; gx <= gxmax; ++gx) {
                    double ddx = xs0 - gx * dx; ddx *= ddx;
                    for (int gy = gymin; gy <= gymax; ++gy) {
                        double ddy = xs1 - gy * dx; ddy *= ddy;
                        double r = sqrt(ddx + ddy);
                        if (r > hs) continue;
                        tot += spline_2d(r * hinv);
                    }
                }
                if (tot == 0.0) continue;
                for (int gx = gxmin; gx <= gxmax; ++gx) {
                    double ddx = xs0 - gx * dx; ddx *= ddx;
                    for (int gy = gymin; gy <= gymax; ++gy) {
                        double ddy = xs1 - gy * dx; ddy *= ddy;
                        double r = sqrt(ddx + ddy);
                        if (r > hs) continue;
                        g[(size_t)gx * res + gy] += spline_2d(r * hinv) * f[i] / tot;
                    }
                }
            }
        }
    }
    double scale = conservative ? 1.0 / (dx * dx) : 1.0;
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < (int64_t)cells; ++c) {
        double s = 0.0;
        for (int t = 0; t < nt; ++t) s += priv[(size_t)t * cells + c];
        grid[c] = s * scale;
    }
    free(priv);
}

/*
 * Exact neighbour-set decision used as the parity rule: given candidate
 * neighbours (a superset, e.g. cKDTree's k+extra nearest), keep the k smallest
 * by (d2, index) where d2 = (dx*dx + dy*dy) + dz*dz in FP64 without
 * contraction, dx = pos[j] - pos[i] (nearest image when boxsize > 0).
 * Writes ngb (Nq, k) int64 and the FP64 distances (Nq, k), ascending.
 */
/* src/meshoid/kernel_density.py:71-78 (kernel3d): 3-D normalised spline,
 * extended by 0 beyond its support q <= 1 (the reference leaves it unassigned
 * there, while the 3-D deposits below evaluate it on every node of a
 * particle's bounding cube). */
static inline double spline_3d(double q) {
    double k;
    if (q <= 0.5) {
        k = 1.0 - 6.0 * q * q * (1.0 - q);
    } else if (q <= 1.0) {
        double a = 1.0 - q;
        k = 2.0 * a * a * a;
    } else {
        k = 0.0;
    }
    return k * 2.546479089470325;
}

/* Python's non-negative modulo */
static inline int pmod(int a, int m) { return ((a % m) + m) % m; }

/* GridDensity (src/meshoid/grid_deposition.py:534-600): per particle, the
 * kernel weights of the nodes g*dx of its bounding cube (clipped to the grid
 * without a box, wrapped modulo res with one) are normalised to 1 and the
 * particle's f is spread by them; the grid is divided by dx^3.  Serial (the
 * reference is serial too). */
void orc_grid_density(const double *f, const double *x, const double *h, int64_t n, const double *center,
                      double size, int res, double box_size, double *grid) {
    const double dx = size / (double)(res - 1);
    const size_t cells = (size_t)res * res * res;
    for (size_t c = 0; c < cells; ++c) grid[c] = 0.0;
    int cap = 0;
    double *kval = NULL;
    for (int64_t i = 0; i < n; ++i) {
        double xs[3];
        for (int d = 0; d < 3; ++d) xs[d] = x[i * 3 + d] - center[d] + size / 2 - dx / 2;
        const double hs = h[i], hinv = 1.0 / hs;
        int lo[3], hi[3];
        for (int d = 0; d < 3; ++d) {
            lo[d] = (int)((xs[d] - hs) / dx + 1);
            hi[d] = (int)((xs[d] + hs) / dx);
            if (box_size < 0) {
                if (lo[d] < 0) lo[d] = 0;
                if (hi[d] > res - 1) hi[d] = res - 1;
            }
        }
        const int nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
        if (nx <= 0 || ny <= 0 || nz <= 0) continue;
        const int cnt = nx * ny * nz;
        if (cnt > cap) {
            cap = cnt;
            kval = (double *)realloc(kval, sizeof(double) * (size_t)cap);
        }
        double total = 0.0;
        int j = 0;
        for (int gx = lo[0]; gx <= hi[0]; ++gx) {
            double ddx = xs[0] - gx * dx; ddx *= ddx;
            for (int gy = lo[1]; gy <= hi[1]; ++gy) {
                double ddy = xs[1] - gy * dx; ddy *= ddy;
                for (int gz = lo[2]; gz <= hi[2]; ++gz) {
                    double ddz = xs[2] - gz * dx; ddz *= ddz;
                    const double k = spline_3d(sqrt(ddx + ddy + ddz) * hinv);
                    total += k;
                    kval[j++] = k;
                }
            }
        }
        if (!(total > 0)) continue;
        j = 0;
        for (int gx = lo[0]; gx <= hi[0]; ++gx)
            for (int gy = lo[1]; gy <= hi[1]; ++gy)
                for (int gz = lo[2]; gz <= hi[2]; ++gz) {
                    const size_t c = ((size_t)pmod(gx, res) * res + pmod(gy, res)) * res + pmod(gz, res);
                    grid[c] += f[i] * kval[j++] / total;
                }
    }
    free(kval);
    const double v = dx * dx * dx;
    for (size_t c = 0; c < cells; ++c) grid[c] /= v;
}

/* Grid_PPZ_DataCube (src/meshoid/grid_deposition.py:339-392): column nodes
 * g*dx in the plane, z nodes g*dz, kernel3d of the anisotropic distance, f /
 * (h^2 h_z) per particle; ranges clipped to the cube. */
void orc_ppz_cube(const double *f, const double *x, const double *h, const double *z, const double *hz, int64_t n,
                  const double *center, double size_xy, double size_z, int res_xy, int res_z, double *grid) {
    const double dx = size_xy / (double)(res_xy - 1), dz = size_z / (double)(res_z - 1);
    const size_t cells = (size_t)res_xy * res_xy * res_z;
    for (size_t c = 0; c < cells; ++c) grid[c] = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        const double x0 = x[i * 3 + 0] - center[0] + size_xy / 2, x1 = x[i * 3 + 1] - center[1] + size_xy / 2;
        const double zs = z[i] - center[2] + size_z / 2;
        const double hs = h[i], hzs = hz[i];
        const double hinvsq = 1 / (hs * hs), hzinvsq = 1 / (hzs * hzs);
        const double fd = f[i] / (hs * hs * hzs);
        int gxmin = (int)((x0 - hs) / dx + 1); if (gxmin < 0) gxmin = 0;
        int gxmax = (int)((x0 + hs) / dx); if (gxmax > res_xy - 1) gxmax = res_xy - 1;
        int gymin = (int)((x1 - hs) / dx + 1); if (gymin < 0) gymin = 0;
        int gymax = (int)((x1 + hs) / dx); if (gymax > res_xy - 1) gymax = res_xy - 1;
        int gzmin = (int)((zs - hzs) / dz + 1); if (gzmin < 0) gzmin = 0;
        int gzmax = (int)((zs + hzs) / dz); if (gzmax > res_z - 1) gzmax = res_z - 1;
        for (int gx = gxmin; gx <= gxmax; ++gx) {
            double ddx = x0 - gx * dx; ddx *= ddx;
            for (int gy = gymin; gy <= gymax; ++gy) {
                double ddy = x1 - gy * dx; ddy *= ddy;
                const double q2 = (ddx + ddy) * hinvsq;
                for (int gz = gzmin; gz <= gzmax; ++gz) {
                    double ddz = zs - gz * dz; ddz *= ddz;
                    grid[((size_t)gx * res_xy + gy) * res_z + gz] += spline_3d(sqrt(q2 + ddz * hzinvsq)) * fd;
                }
            }
        }
    }
}

/* WeightedGridInterp3D (src/meshoid/grid_deposition.py:439-531): cell-centre
 * nodes linspace(dx/2 - size/2, size/2 - dx/2, res) (dx = size/(res-1)), per
 * particle kernel weights normalised to 1 times wt spread into a value grid
 * (times f) and a weight grid; result = value / weight, and a cell without
 * weight takes the f of the nearest particle (first in index order). */
void orc_weighted_interp3d(const double *f, const double *wt, const double *x, const double *h, int64_t n,
                           const double *center, double size, int res, double *result) {
    const double dx = size / (double)(res - 1);
    double *coord = (double *)malloc(sizeof(double) * (size_t)res);
    const double start = dx / 2 - size / 2, stop = size / 2 - dx / 2;
    const double step = (stop - start) / (double)(res - 1);
    for (int i = 0; i < res; ++i) coord[i] = (double)i * step + start;
    coord[res - 1] = stop;
    const size_t cells = (size_t)res * res * res;
    double *num = (double *)calloc(cells, sizeof(double)), *den = (double *)calloc(cells, sizeof(double));
    int cap = 0;
    double *kval = NULL;
    for (int64_t i = 0; i < n; ++i) {
        double xs[3], gi[3];
        for (int d = 0; d < 3; ++d) {
            xs[d] = x[i * 3 + d] - center[d];
            gi[d] = (xs[d] + size / 2) / dx - 0.5;
        }
        const double hs = h[i], hinv = 1 / hs, hs_dx = hs / dx;
        int lo[3], hi[3];
        for (int d = 0; d < 3; ++d) {
            lo[d] = (int)(gi[d] - hs_dx + 1); if (lo[d] < 0) lo[d] = 0;
            hi[d] = (int)(gi[d] + hs_dx); if (hi[d] > res - 1) hi[d] = res - 1;
        }
        const int nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
        if (nx <= 0 || ny <= 0 || nz <= 0) continue;
        const int cnt = nx * ny * nz;
        if (cnt > cap) {
            cap = cnt;
            kval = (double *)realloc(kval, sizeof(double) * (size_t)cap);
        }
        double total = 0.0;
        int j = 0;
        for (int gx = lo[0]; gx <= hi[0]; ++gx) {
            double ddx = xs[0] - coord[gx]; ddx *= ddx;
            for (int gy = lo[1]; gy <= hi[1]; ++gy) {
                double ddy = xs[1] - coord[gy]; ddy *= ddy;
                for (int gz = lo[2]; gz <= hi[2]; ++gz) {
                    double ddz = xs[2] - coord[gz]; ddz *= ddz;
                    const double k = spline_3d(sqrt(ddx + ddy + ddz) * hinv);
                    total += k;
                    kval[j++] = k;
                }
            }
        }
        if (!(total > 0)) continue;
        j = 0;
        for (int gx = lo[0]; gx <= hi[0]; ++gx)
            for (int gy = lo[1]; gy <= hi[1]; ++gy)
                for (int gz = lo[2]; gz <= hi[2]; ++gz) {
                    const double k = kval[j++];
                    const size_t c = ((size_t)gx * res + gy) * res + gz;
                    num[c] += f[i] * k * wt[i] / total;
                    den[c] += k * wt[i] / total;
                }
    }
    for (int a = 0; a < res; ++a)
        for (int b = 0; b < res; ++b)
            for (int c3 = 0; c3 < res; ++c3) {
                const size_t c = ((size_t)a * res + b) * res + c3;
                if (den[c] != 0.0) {
                    result[c] = num[c] / den[c];
                    continue;
                }
                const double pc[3] = {coord[a], coord[b], coord[c3]};
                double best = 1e100;
                int64_t bi = -1;
                for (int64_t p = 0; p < n; ++p) {
                    double dd = 0.0;
                    for (int d = 0; d < 3; ++d) {
                        const double t = (x[p * 3 + d] - center[d]) - pc[d];
                        dd += t * t;
                    }
                    if (dd < best) {
                        best = dd;
                        bi = p;
                    }
                }
                result[c] = bi >= 0 ? f[bi] : NAN;
            }
    free(kval);
    free(coord);
    free(num);
    free(den);
}

/* radtransfer_singlethread (src/meshoid/radiation/radtransfer.py:87-200):
 * particles from the largest z to the smallest (relative to the centre; ties
 * by index), each one attenuating and emitting into the pixels of its
 * footprint (nodes g * dx, dx = L / (res - 1), from centre - L/2; h at least
 * dx): tau = kappa kernel2d(r / h) m / h^2, I <- exp(-tau) I - expm1(-tau)
 * j / (4 pi kappa + 1e-100).  I starts at i0 (bands, or NULL for 0). */
static const double *rt_z;
static int rt_cmp(const void *a, const void *b) {
    const int64_t i = *(const int64_t *)a, k = *(const int64_t *)b;
    if (rt_z[i] > rt_z[k]) return -1;
    if (rt_z[i] < rt_z[k]) return 1;
    return i < k ? -1 : (i > k);
}

void orc_radtransfer(const double *j, const double *m, const double *kappa, const double *x, const double *h,
                     int64_t n, int bands, int res, double L, const double *center, const double *i0, double *inten,
                     double *taumap) {
    const double dx = L / (double)(res - 1);
    const size_t cells = (size_t)res * res * bands;
    for (size_t c = 0; c < cells; ++c) {
        inten[c] = i0 ? i0[c % bands] : 0.0;
        taumap[c] = 0.0;
    }
    double *z = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    int64_t *order = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) {
        z[i] = x[i * 3 + 2] - center[2];
        order[i] = i;
    }
    rt_z = z;
    qsort(order, (size_t)n, sizeof(int64_t), rt_cmp);
    const double pi = 3.14159265358979323846;
    for (int64_t r = 0; r < n; ++r) {
        const int64_t i = order[r];
        const double xs0 = x[i * 3 + 0] - center[0] + L / 2, xs1 = x[i * 3 + 1] - center[1] + L / 2;
        const double hs = h[i] > dx ? h[i] : dx;
        if (hs == 0 || m[i] == 0) continue;
        const double mh2 = m[i] / (hs * hs);
        int gxmin = (int)((xs0 - hs) / dx + 1); if (gxmin < 0) gxmin = 0;
        int gxmax = (int)((xs0 + hs) / dx); if (gxmax > res - 1) gxmax = res - 1;
        int gymin = (int)((xs1 - hs) / dx + 1); if (gymin < 0) gymin = 0;
        int gymax = (int)((xs1 + hs) / dx); if (gymax > res - 1) gymax = res - 1;
        for (int gx = gxmin; gx <= gxmax; ++gx) {
            double ddx = xs0 - gx * dx; ddx *= ddx;
            for (int gy = gymin; gy <= gymax; ++gy) {
                double ddy = xs1 - gy * dx; ddy *= ddy;
                const double rr = ddx + ddy;
                if (rr > hs * hs) continue;
                const double ker = spline_2d(sqrt(rr) / hs);
                for (int b = 0; b < bands; ++b) {
                    const double kap = kappa[i * bands + b];
                    const double src = j[i * bands + b] / (4 * pi * kap + 1e-100);
                    const double tau = kap * ker * mh2;
                    const size_t c = ((size_t)gx * res + gy) * bands + b;
                    taumap[c] += tau;
                    inten[c] = exp(-tau) * inten[c] + (-expm1(-tau)) * src;
                }
            }
        }
    }
    free(z);
    free(order);
}

void orc_knn_decide(const double *pos, int dim, const int64_t *queries, int64_t nq,
                    const int64_t *cand, int kc, int k, double boxsize,
                    int64_t *ngb_out, double *dist_out) {
#pragma omp parallel
    {
        double *d2 = (double *)malloc(sizeof(double) * kc);
        int64_t *id = (int64_t *)malloc(sizeof(int64_t) * kc);
#pragma omp for schedule(static)
        for (int64_t i = 0; i < nq; ++i) {
            int64_t q = queries[i];
            int m = 0;
            for (int c = 0; c < kc; ++c) {
                int64_t j = cand[i * kc + c];
                if (j < 0) continue;
                double s = 0.0;
                for (int a = 0; a < dim; ++a) {
                    double d = pos[j * dim + a] - pos[q * dim + a];
                    if (boxsize > 0) d = nearest_image(d, boxsize);
                    double dd = d * d;
                    s = s + dd;
                }
                d2[m] = s; id[m] = j; ++m;
            }
            /* insertion sort by (d2, idx): kc is small */
            for (int a = 1; a < m; ++a) {
                double dv = d2[a]; int64_t iv = id[a]; int b = a - 1;
                while (b >= 0 && (d2[b] > dv || (d2[b] == dv && id[b] > iv))) {
                    d2[b + 1] = d2[b]; id[b + 1] = id[b]; --b;
                }
                d2[b + 1] = dv; id[b + 1] = iv;
            }
            for (int c = 0; c < k; ++c) {
                ngb_out[i * k + c] = c < m ? id[c] : -1;
                dist_out[i * k + c] = c < m ? sqrt(d2[c]) : INFINITY;
            }
        }
        free(d2); free(id);
    }
}
