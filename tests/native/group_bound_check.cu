// Host check of the first search pass's distance error bound (k_knn_group in
// meshoid_gb300/csrc/mg_knn.cu): offsets from the block centre are formed from
// the FP32 hi/lo position split as (hi - centre) + lo, squared distances by
// the pass's FP32 expression, and the set is exact when every candidate's
// FP32 distance lies within e2 = 1.01 eg + 2e-7 R of the true distance, with
// eg = 1e-6 ehalf + 3e-7 rmax from the block's box.  The box, its margin and
// the centre follow the kernel's arithmetic; the geometries are adversarial
// (blocks far from the frame origin, radii spanning decades inside a block,
// clusters narrower than an FP32 ulp of the position).  Built and run on the
// CPU by tests/test_native_helpers.py.
#include <math.h>
#include <stdint.h>
#include <stdio.h>

static uint64_t rng_state = 0xBF58476D1CE4E5B9ull;
static double urand() {
    rng_state ^= rng_state >> 12;
    rng_state ^= rng_state << 25;
    rng_state ^= rng_state >> 27;
    return (double)((rng_state * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0);
}

// the pass's squared distance between offsets (group_d2: sub, mul, two fma)
static float d2_fp32(const float c[3], const float q[3]) {
    const float dx = c[0] - q[0], dy = c[1] - q[1], dz = c[2] - q[2];
    float d2 = dx * dx;
    d2 = fmaf(dy, dy, d2);
    d2 = fmaf(dz, dz, d2);
    return d2;
}

int main() {
    const int NQ = 128, NC = 256;
    double worst = 0.0;
    long long checked = 0;
    int fails = 0;
    for (int t = 0; t < 4000; ++t) {
        // frame-relative positions in [0, side): the block sits anywhere, its
        // members in a cluster of scale s, radii spanning up to 2x (members) as the pass admits
        const double side = pow(10.0, -3.0 + 6.0 * urand());
        double cen[3];
        for (int d = 0; d < 3; ++d) cen[d] = side * urand();
        const double s = side * pow(10.0, -9.0 * urand());
        const double r0 = s * pow(10.0, -1.0 + 2.0 * urand());
        double X[NQ + NC][3], R[NQ];
        float hi[NQ + NC][3], lo[NQ + NC][3];
        for (int i = 0; i < NQ + NC; ++i)
            for (int d = 0; d < 3; ++d) {
                X[i][d] = cen[d] + s * (2.0 * urand() - 1.0) * (i < NQ ? 1.0 : 1.5);
                hi[i][d] = (float)X[i][d];
                lo[i][d] = (float)(X[i][d] - (double)hi[i][d]);
            }
        float rmin = 3e38f, rmax = 0.0f;
        float Rf[NQ];
        for (int i = 0; i < NQ; ++i) {
            R[i] = r0 * (1.0 + urand());  // within the pass's 2 x rmin member rule
            Rf[i] = (float)R[i];
            rmin = fminf(rmin, Rf[i]);
            rmax = fmaxf(rmax, Rf[i]);
        }
        // the block's box from the hi parts, its margin, centre and half extent
        float blo[3] = {3e38f, 3e38f, 3e38f}, bhi[3] = {-3e38f, -3e38f, -3e38f};
        for (int i = 0; i < NQ; ++i)
            for (int d = 0; d < 3; ++d) {
                blo[d] = fminf(blo[d], hi[i][d] - Rf[i]);
                bhi[d] = fmaxf(bhi[d], hi[i][d] + Rf[i]);
            }
        float xm = 0.0f;
        for (int d = 0; d < 3; ++d) xm = fmaxf(xm, fmaxf(fabsf(blo[d]), fabsf(bhi[d])));
        const float mg = 1e-5f * rmax + 4e-7f * xm + 1e-30f;
        float ctr[3], ehalf = 0.0f;
        for (int d = 0; d < 3; ++d) {
            blo[d] -= mg;
            bhi[d] += mg;
            ctr[d] = 0.5f * (blo[d] + bhi[d]);
            ehalf = fmaxf(ehalf, fmaxf(fabsf(blo[d] - ctr[d]), fabsf(bhi[d] - ctr[d])));
        }
        const float eg = 1e-6f * ehalf + 3e-7f * rmax;
        float off[NQ + NC][3];
        for (int i = 0; i < NQ + NC; ++i)
            for (int d = 0; d < 3; ++d) off[i][d] = (hi[i][d] - ctr[d]) + lo[i][d];
        for (int q = 0; q < NQ; ++q) {
            const float e2 = 1.01f * eg + 2e-7f * Rf[q];
            for (int c = 0; c < NQ + NC; ++c) {
                double dd = 0.0;
                for (int d = 0; d < 3; ++d) {
                    const double v = ((double)hi[c][d] + lo[c][d]) - ((double)hi[q][d] + lo[q][d]);
                    dd += v * v;
                }
                const double d = sqrt(dd);
                if (d > 1.5 * R[q]) continue;  // the bound is claimed for candidates near the sphere
                const double dt = sqrt((double)d2_fp32(off[c], off[q]));
                const double dtf = (double)sqrtf(d2_fp32(off[c], off[q]));
                const double err = fmax(fabs(dt - d), fabs(dtf - d));
                ++checked;
                worst = fmax(worst, err / e2);
                if (err > e2) {
                    if (fails < 10)
                        printf("  side %.3g s %.3g R %.3g: |d~ - d| %.3g above e2 %.3g\n", side, s, R[q], err, e2);
                    ++fails;
                }
            }
        }
    }
    printf("group pass bound: %lld candidate distances, worst |d~ - d| / e2 %.3g, above it %d\n", checked, worst,
           fails);
    printf(fails ? "FAILED\n" : "ok\n");
    return fails ? 1 : 0;
}
