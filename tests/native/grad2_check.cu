// Host check of the float-float order-2 derivative arithmetic
// (meshoid_gb300/csrc/mg_grad2.cuh, mg_ff.cuh) against FP64, on random
// neighbourhoods: balls of 32 points, flattened ones, and tight clusters far
// from the origin (separations ~1e-5 of the coordinates, where FP32
// separations lose the answer), with fields that vary inside the kernel and
// carry a large constant offset (so neighbour differences are ~1e-5 of the
// values: the three-plane split keeps them).  Checks
//   * hsml_polish_ff against an FP64 Newton root of HsmlIter's equation;
//   * the float-float moments / right-hand sides / Cholesky factor and solve
//     (g2_basis, g2_moments_add, g2_rhs_add, g2_chol_ff, g2_solve_ff) against
//     an FP64 least-squares solve at the same h, on rows with FP64 condition
//     < 1e7 (flattened neighbourhoods reach ~1e7);
//   * g2_factor64 / g2_solve64 against the same FP64 solve.
// Built and run on the CPU by tests/test_native_helpers.py; prints one line
// per check and exits non-zero on a failure.
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include "mg_grad2.cuh"
#include "mg_refine.cuh"

using namespace mg;

static uint64_t rng_state = 0xD1B54A32D192ED03ull;
static double urand() {
    rng_state ^= rng_state >> 12;
    rng_state ^= rng_state << 25;
    rng_state ^= rng_state >> 27;
    return (double)((rng_state * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0);
}
static double nrand() {
    const double u = urand() + 1e-300, v = urand();
    return sqrt(-2.0 * log(u)) * cos(6.283185307179586 * v);
}
static void split2(double v, float &h, float &l) {
    h = (float)v;
    l = (float)(v - (double)h);
}
static void split3(double v, float &h, float &m, float &l) {
    h = (float)v;
    const double r = v - (double)h;
    m = (float)r;
    l = (float)(r - (double)m);
}
static double w64(double q) {
    return q <= 0.5 ? 1.0 - 6.0 * q * q + 6.0 * q * q * q : (q <= 1.0 ? 2.0 * (1.0 - q) * (1.0 - q) * (1.0 - q) : 0.0);
}

// FP64 Gauss-Jordan with partial pivoting; returns false when singular
static bool solve64(int n, double A[9][9], double b[9]) {
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (fabs(A[r][c]) > fabs(A[piv][c])) piv = r;
        if (fabs(A[piv][c]) < 1e-300) return false;
        for (int k = 0; k < n; ++k) {
            const double t = A[c][k];
            A[c][k] = A[piv][k];
            A[piv][k] = t;
        }
        const double t = b[c];
        b[c] = b[piv];
        b[piv] = t;
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            const double f = A[r][c] / A[c][c];
            for (int k = c; k < n; ++k) A[r][k] -= f * A[c][k];
            b[r] -= f * b[c];
        }
    }
    for (int c = 0; c < n; ++c) b[c] /= A[c][c];
    return true;
}

// power iteration bounds for the 2-norm condition number of a symmetric PD matrix
static double cond64(int n, const double A[9][9]) {
    double B[9][9];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) B[i][j] = A[i][j];
    double v[9], lmax = 0.0;
    for (int i = 0; i < n; ++i) v[i] = 1.0 + 0.1 * i;
    for (int it = 0; it < 200; ++it) {
        double w[9], nrm = 0.0;
        for (int i = 0; i < n; ++i) {
            w[i] = 0.0;
            for (int j = 0; j < n; ++j) w[i] += B[i][j] * v[j];
            nrm += w[i] * w[i];
        }
        nrm = sqrt(nrm);
        for (int i = 0; i < n; ++i) v[i] = w[i] / nrm;
        lmax = nrm;
    }
    // smallest eigenvalue: inverse iteration through repeated solves
    for (int i = 0; i < n; ++i) v[i] = 1.0 - 0.07 * i;
    double lmin = 0.0;
    for (int it = 0; it < 60; ++it) {
        double C[9][9], x[9];
        for (int i = 0; i < n; ++i) {
            x[i] = v[i];
            for (int j = 0; j < n; ++j) C[i][j] = B[i][j];
        }
        if (!solve64(n, C, x)) return 1e300;
        double nrm = 0.0;
        for (int i = 0; i < n; ++i) nrm += x[i] * x[i];
        nrm = sqrt(nrm);
        for (int i = 0; i < n; ++i) v[i] = x[i] / nrm;
        lmin = 1.0 / nrm;
    }
    return lmax / lmin;
}

template <int DIM>
static int run(const char *name, int geometry, int reps, double &worst_x, double &worst_h, double &worst_64,
               int &checked) {
    constexpr int ND = G2<DIM>::ND, NM = G2<DIM>::NM, K = 32;
    int fails = 0;
    for (int rep = 0; rep < reps; ++rep) {
        // query position and neighbours (FP64)
        const double scale = geometry == 2 ? 1e-5 : 1.0;
        double q0[3] = {0.0, 0.0, 0.0};
        for (int c = 0; c < DIM; ++c) q0[c] = geometry == 2 ? 0.7 + 0.2 * urand() : 2.0 * urand() - 1.0;
        double P[K][3], dist[K];
        for (int j = 0; j < K; ++j) {
            for (int c = 0; c < 3; ++c) P[j][c] = q0[c];
            if (j == 0) continue;  // the query itself
            for (int c = 0; c < DIM; ++c) {
                double d = scale * nrand();
                if (geometry == 1 && c == DIM - 1) d *= rep % 2 ? 0.2 : 0.03;  // flattened
                P[j][c] = q0[c] + d;
            }
        }
        for (int j = 0; j < K; ++j) {
            double r2 = 0.0;
            for (int c = 0; c < DIM; ++c) r2 += (P[j][c] - q0[c]) * (P[j][c] - q0[c]);
            dist[j] = sqrt(r2);
        }
        // FP64 root of HsmlIter's equation: bisection on [second distance,
        // 2 x largest] (n - k changes sign there), then Newton polish
        const double norm = DIM == 3 ? 32.0 / 3.0 : (DIM == 2 ? 40.0 / 7.0 : 8.0 / 3.0);
        double dmax = 0.0, dmin = 1e300;
        for (int j = 0; j < K; ++j) {
            dmax = fmax(dmax, dist[j]);
            if (dist[j] > 0.0) dmin = fmin(dmin, dist[j]);
        }
        auto nk = [&](double hh, double &dn) {
            double n = 0.0;
            dn = 0.0;
            for (int j = 0; j < K; ++j) {
                const double q = dist[j] / hh;
                n += w64(q);
                const double dw = q <= 0.5 ? q * (18.0 * q - 12.0) : (q <= 1.0 ? -6.0 * (1.0 - q) * (1.0 - q) : 0.0);
                dn += -dw * q / hh;
            }
            dn *= norm;
            return norm * n - K;
        };
        double lo = dmin, hi = 2.0 * dmax, dn;
        for (int it = 0; it < 200; ++it) {
            const double mid = 0.5 * (lo + hi);
            (nk(mid, dn) > 0.0 ? hi : lo) = mid;
        }
        double h = 0.5 * (lo + hi);
        for (int it = 0; it < 3; ++it) h -= nk(h, dn) / dn;
        // the FP32 solve's h, then the float-float polish from hi/lo positions
        float qh[3] = {0, 0, 0}, ql[3] = {0, 0, 0};
        for (int c = 0; c < DIM; ++c) split2(q0[c], qh[c], ql[c]);
        auto sep = [&](int j, ff d[3]) {
            for (int c = 0; c < 3; ++c) d[c] = ff{0.0f, 0.0f};
            for (int c = 0; c < DIM; ++c) {
                float bh, bl, lo;
                split2(P[j][c], bh, bl);
                const float s = sep1_ff(bh, qh[c], bl, ql[c], lo);
                d[c] = ff{s, lo};
            }
        };
        const float h32 = (float)(h * (1.0 + 3e-7 * (2.0 * urand() - 1.0)));
        const ff hp = hsml_polish_ff<DIM>(
            [&](int j) {
                ff d[3];
                sep(j, d);
                ff r2 = ff{0.0f, 0.0f};
                for (int c = 0; c < DIM; ++c) r2 = ff_add(r2, ff_sqr(d[c]));
                return ff_sqrt(r2);
            },
            K, h32);
        const double hpd = (double)hp.hi + (double)hp.lo;
        // the float-float distances carry 2^-48 of the coordinates (hi/lo
        // split): for a cluster far from the origin that is the limit
        double qmag = 0.0;
        for (int c = 0; c < DIM; ++c) qmag = fmax(qmag, fabs(q0[c]));
        worst_h = fmax(worst_h, fabs(hpd / h - 1.0));
        if (fabs(hpd / h - 1.0) > 1e-10 + 1e-14 * qmag / h) {
            if (fails < 5) printf("  %s rep %d: h %.17g polished %.17g\n", name, rep, h, hpd);
            ++fails;
        }
        // fields: offset + oscillation inside the kernel + a linear part
        constexpr int F = 3;
        double fv[F][K];
        const double kw = 6.0 / h;
        for (int u = 0; u < F; ++u)
            for (int j = 0; j < K; ++j) {
                const double x = (P[j][0] - q0[0]), y = DIM > 1 ? P[j][1] - q0[1] : 0.0;
                fv[u][j] = (u == 0 ? 1e3 : (u == 1 ? 1.0 : 0.0)) + sin(kw * x + 0.3 * u) * cos(kw * y) + 0.5 * x / h;
            }
        // FP64 reference at the polished h (the same h the float-float path uses)
        double A64[9][9] = {}, B64[F][9] = {};
        const double hinv64 = 1.0 / hpd;
        for (int j = 0; j < K; ++j) {
            double a[ND], d[3] = {0, 0, 0};
            for (int c = 0; c < DIM; ++c) d[c] = P[j][c] - q0[c];
            const double w = g2_basis64<DIM>(d, hinv64, true, a);
            if (w == 0.0) continue;
            for (int i = 0; i < ND; ++i)
                for (int l = 0; l < ND; ++l) A64[i][l] += w * a[i] * a[l];
            for (int u = 0; u < F; ++u)
                for (int i = 0; i < ND; ++i) B64[u][i] += w * a[i] * (fv[u][j] - fv[u][0]);
        }
        const double cnd = cond64(ND, A64);
        // FP64 packed path (g2_factor64 / g2_solve64)
        double Ap[NM];
        for (int i = 0; i < ND; ++i)
            for (int l = 0; l <= i; ++l) Ap[g2_idx(i, l)] = A64[i][l];
        g2_factor64<ND>(Ap);  // positive definite here (cond < 1e7 rows are checked)
        // float-float path
        const ff hinv = ff_recip2(hp.hi, hp.lo);
        ff M[NM], b[F][ND];
        for (int i = 0; i < NM; ++i) M[i] = ff{0.0f, 0.0f};
        for (int u = 0; u < F; ++u)
            for (int m = 0; m < ND; ++m) b[u][m] = ff{0.0f, 0.0f};
        float f0[F][3];
        for (int u = 0; u < F; ++u) split3(fv[u][0], f0[u][0], f0[u][1], f0[u][2]);
        for (int j = 0; j < K; ++j) {
            ff d[3], a[ND], wa[ND];
            sep(j, d);
            if (!g2_basis<DIM>(d, hinv, true, a, wa)) continue;
            g2_moments_add<DIM>(M, a, wa);
            for (int u = 0; u < F; ++u) {
                float fh, fm, fl;
                split3(fv[u][j], fh, fm, fl);
                g2_rhs_add<DIM>(b[u], wa, ff_diff3(fh, fm, fl, f0[u][0], f0[u][1], f0[u][2]));
            }
        }
        for (int i = 0; i < NM; ++i) M[i] = ff_norm(M[i]);
        const bool chol = g2_chol_ff<ND>(M);
        if (!(cnd < 1e7) || !chol) continue;
        ++checked;
        for (int u = 0; u < F; ++u) {
            double x64[9], A[9][9];
            for (int i = 0; i < ND; ++i) {
                x64[i] = B64[u][i];
                for (int l = 0; l < ND; ++l) A[i][l] = A64[i][l];
            }
            solve64(ND, A, x64);
            double xp[ND];
            for (int i = 0; i < ND; ++i) xp[i] = B64[u][i];
            g2_solve64<ND>(Ap, xp);
            ff bn[ND];
            for (int m = 0; m < ND; ++m) bn[m] = ff_norm(b[u][m]);
            g2_solve_ff<ND>([&](int i) { return M[i]; }, bn);
            double e1 = 0, n1 = 0, e2 = 0, n2 = 0, p1 = 0, p2 = 0;
            for (int m = 0; m < ND; ++m) {
                const double e = ((double)bn[m].hi + (double)bn[m].lo) - x64[m], ep = xp[m] - x64[m];
                if (m < DIM) {
                    e1 += e * e;
                    p1 += ep * ep;
                    n1 += x64[m] * x64[m];
                } else {
                    e2 += e * e;
                    p2 += ep * ep;
                    n2 += x64[m] * x64[m];
                }
            }
            const double err = fmax(sqrt(e1 / n1), sqrt(e2 / n2));
            const double err64 = fmax(sqrt(p1 / n1), sqrt(p2 / n2));
            worst_x = fmax(worst_x, err);
            worst_64 = fmax(worst_64, err64);
            if (err > 2e-7 || err64 > 1e-9 * fmax(1.0, cnd / 1e5)) {
                if (fails < 5)
                    printf("  %s rep %d field %d: cond %.3g err %.3g err64 %.3g\n", name, rep, u, cnd, err, err64);
                ++fails;
            }
        }
    }
    return fails;
}

int main() {
    int fails = 0;
    const char *names[] = {"ball", "flattened", "tight cluster far from the origin"};
    for (int geom = 0; geom < 3; ++geom) {
        double wx = 0, wh = 0, w64v = 0;
        int checked = 0;
        fails += run<3>(names[geom], geom, 400, wx, wh, w64v, checked);
        printf("3-D %s: rows checked %d, float-float worst %.3g, FP64 packed worst %.3g, polished h worst %.3g\n",
               names[geom], checked, wx, w64v, wh);
    }
    {
        double wx = 0, wh = 0, w64v = 0;
        int checked = 0;
        fails += run<2>("2-D ball", 0, 300, wx, wh, w64v, checked);
        printf("2-D ball: rows checked %d, float-float worst %.3g, FP64 packed worst %.3g, polished h worst %.3g\n",
               checked, wx, w64v, wh);
    }
    if (fails) {
        printf("FAILED %d\n", fails);
        return 1;
    }
    printf("ok\n");
    return 0;
}
