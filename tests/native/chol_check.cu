// Host check of the derivative sweep's FP32 factor, solve and condition
// estimate (meshoid_gb300/csrc/mg_chol.cuh) on moment matrices of random
// neighbourhoods, flattened to raise their condition numbers, against FP64
// (Jacobi eigenvalues, Cholesky solve).  The estimate decides which rows the
// sweep re-solves in FP64, so it must not fall below the true 2-norm
// condition number.  Built and run on the CPU by tests/test_native_helpers.py.
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include "mg_chol.cuh"

using namespace mg;

static uint64_t rng_state = 0xD1B54A32D192ED03ull;
static double urand() {
    rng_state ^= rng_state >> 12;
    rng_state ^= rng_state << 25;
    rng_state ^= rng_state >> 27;
    return (double)((rng_state * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0);
}

// eigenvalues of a symmetric n x n matrix (cyclic Jacobi, FP64)
static void eig_sym(int n, double A[9][9], double *ev) {
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = i + 1; j < n; ++j) off += A[i][j] * A[i][j];
        if (off < 1e-300) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                if (fabs(A[p][q]) < 1e-300) continue;
                const double th = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {
                    const double akp = A[k][p], akq = A[k][q];
                    A[k][p] = c * akp - s * akq;
                    A[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = c * apk - s * aqk;
                    A[q][k] = s * apk + c * aqk;
                }
            }
    }
    for (int i = 0; i < n; ++i) ev[i] = A[i][i];
}

// basis of the sweep: dim first-order terms, then (order 2) squares / 2 and cross terms
static int basis(int dim, int order, const double x[3], double *a) {
    int m = 0;
    for (int d = 0; d < dim; ++d) a[m++] = x[d];
    if (order == 2) {
        for (int d = 0; d < dim; ++d) a[m++] = 0.5 * x[d] * x[d];
        if (dim == 2) a[m++] = x[0] * x[1];
        if (dim == 3) { a[m++] = x[0] * x[1]; a[m++] = x[1] * x[2]; a[m++] = x[2] * x[0]; }
    }
    return m;
}

template <int N>
static int run(int dim, int order, int cases, double &worst_under, double &worst_solve, int &estimate_low) {
    constexpr int NM = N * (N + 1) / 2;
    int fails = 0;
    for (int t = 0; t < cases; ++t) {
        // 32 neighbours in the unit ball, squashed along the last axis to raise the condition
        const double squash = pow(10.0, -3.0 * urand());
        double A[9][9] = {};
        for (int j = 0; j < 32; ++j) {
            double x[3] = {0, 0, 0}, r2;
            do {
                r2 = 0.0;
                for (int d = 0; d < dim; ++d) { x[d] = 2.0 * urand() - 1.0; r2 += x[d] * x[d]; }
            } while (r2 > 1.0);
            x[dim - 1] *= squash;
            const double q = sqrt(r2);
            const double w = q <= 0.5 ? 1 - 6 * q * q + 6 * q * q * q : 2 * (1 - q) * (1 - q) * (1 - q);
            double a[9];
            basis(dim, order, x, a);
            for (int i = 0; i < N; ++i)
                for (int k = 0; k < N; ++k) A[i][k] += w * a[i] * a[k];
        }
        float M[NM], L[NM];
        for (int i = 0; i < N; ++i)
            for (int k = 0; k <= i; ++k) M[i * (i + 1) / 2 + k] = L[i * (i + 1) / 2 + k] = (float)A[i][k];
        double Ac[9][9], ev[9];
        for (int i = 0; i < N; ++i)
            for (int k = 0; k < N; ++k) Ac[i][k] = (double)M[i * (i + 1) / 2 + (k <= i ? k : 0)];
        for (int i = 0; i < N; ++i)
            for (int k = 0; k < N; ++k) Ac[i][k] = k <= i ? (double)M[i * (i + 1) / 2 + k] : (double)M[k * (k + 1) / 2 + i];
        eig_sym(N, Ac, ev);
        double emin = 1e300, emax = 0.0;
        for (int i = 0; i < N; ++i) { emin = fmin(emin, ev[i]); emax = fmax(emax, ev[i]); }
        const double cond = emax / emin;
        if (!(emin > 0.0) || cond > 1e7) continue;  // the sweep re-solves these whatever the estimate
        if (!cholesky<N>(L)) {
            // a failed factor queues the row for FP64: never harmful, count it only when cond is small
            if (cond < 1e4) { printf("  N %d: factor failed at cond %.3g\n", N, cond); ++fails; }
            continue;
        }
        const float est = cond_estimate<N>(M, L);
        const double ratio = est / cond;  // must not be far below 1
        worst_under = fmin(worst_under, ratio);
        if (ratio < 0.5) {
            ++estimate_low;
            if (cond > 30.0 || est < 30.0) {  // only an underestimate across the order-1 threshold matters
                if (fails < 10) printf("  N %d: estimate %.4g below cond %.4g\n", N, est, cond);
                ++fails;
            }
        }
        // solve against FP64 for a random right-hand side
        double b[9], xd[9];
        float xf[9];
        for (int i = 0; i < N; ++i) { b[i] = 2.0 * urand() - 1.0; xf[i] = (float)b[i]; }
        chol_solve<N>(L, xf);
        // FP64 reference: Gaussian elimination on the FP32 matrix's exact values
        double G[9][10];
        for (int i = 0; i < N; ++i) {
            for (int k = 0; k < N; ++k) G[i][k] = k <= i ? (double)M[i * (i + 1) / 2 + k] : (double)M[k * (k + 1) / 2 + i];
            G[i][N] = (double)(float)b[i];
        }
        for (int c = 0; c < N; ++c) {
            int pv = c;
            for (int r = c + 1; r < N; ++r) if (fabs(G[r][c]) > fabs(G[pv][c])) pv = r;
            for (int k = 0; k <= N; ++k) { const double tmp = G[c][k]; G[c][k] = G[pv][k]; G[pv][k] = tmp; }
            for (int r = 0; r < N; ++r) {
                if (r == c) continue;
                const double f = G[r][c] / G[c][c];
                for (int k = c; k <= N; ++k) G[r][k] -= f * G[c][k];
            }
        }
        double nx = 0.0, ne = 0.0;
        for (int i = 0; i < N; ++i) {
            xd[i] = G[i][N] / G[i][i];
            nx += xd[i] * xd[i];
            ne += (xf[i] - xd[i]) * (xf[i] - xd[i]);
        }
        // FP32 Cholesky: forward error within a modest multiple of 2^-24 cond
        const double rel = sqrt(ne / nx) / (ldexp(1.0, -24) * cond * N);
        worst_solve = fmax(worst_solve, rel);
        if (rel > 4.0) {
            if (fails < 10) printf("  N %d: solve error %.3g x (2^-24 cond N) at cond %.3g\n", N, rel, cond);
            ++fails;
        }
    }
    return fails;
}

int main() {
    int fails = 0;
    const struct { int dim, order; } cfg[] = {{2, 1}, {3, 1}, {2, 2}, {3, 2}};
    for (const auto &c : cfg) {
        double worst_under = 1e300, worst_solve = 0.0;
        int low = 0, f = 0;
        if (c.dim == 2 && c.order == 1) f = run<2>(2, 1, 20000, worst_under, worst_solve, low);
        if (c.dim == 3 && c.order == 1) f = run<3>(3, 1, 20000, worst_under, worst_solve, low);
        if (c.dim == 2 && c.order == 2) f = run<5>(2, 2, 20000, worst_under, worst_solve, low);
        if (c.dim == 3 && c.order == 2) f = run<9>(3, 2, 20000, worst_under, worst_solve, low);
        printf("dim %d order %d: smallest estimate / cond %.3g (%d below 0.5), worst solve error %.3g x "
               "(2^-24 cond N), failures %d\n", c.dim, c.order, worst_under, low, worst_solve, f);
        fails += f;
    }
    printf(fails ? "FAILED\n" : "ok\n");
    return fails ? 1 : 0;
}
