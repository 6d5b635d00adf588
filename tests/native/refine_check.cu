// Host check of the float-float helpers of the order-2 refinement step
// (meshoid_gb300/csrc/mg_refine.cuh) against FP64, and of their agreement
// with the separations the sweep's first pass uses (sep_hilo, wrap1).
// Built and run on the CPU by tests/test_native_helpers.py; prints one line
// per check and exits non-zero on a failure.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "mg_refine.cuh"

using namespace mg;

static uint64_t rng_state = 0x9E3779B97F4A7C15ull;
static double urand() {  // xorshift64*, uniform in [0, 1)
    rng_state ^= rng_state >> 12;
    rng_state ^= rng_state << 25;
    rng_state ^= rng_state >> 27;
    return (double)((rng_state * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0);
}
static double urange(double a, double b) { return a + (b - a) * urand(); }

static void split(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}
static bool same_bits(float a, float b) { return memcmp(&a, &b, sizeof(float)) == 0; }

static int check_sep() {
    int bad_bits = 0, bad_err = 0;
    double worst = 0.0;
    for (int t = 0; t < 200000; ++t) {
        const double pa = urange(-2.0, 2.0);
        const double off = urange(-1.0, 1.0) * pow(10.0, urange(-7.0, -0.5));
        float ha, la, hb, lb;
        split(pa, ha, la);
        split(pa + off, hb, lb);
        float lo;
        const float d = sep1_ff(hb, ha, lb, la, lo);
        const float4 A = make_float4(ha, 0.f, 0.f, 0.f), Al = make_float4(la, 0.f, 0.f, 0.f);
        const float4 B = make_float4(hb, 0.f, 0.f, 0.f), Bl = make_float4(lb, 0.f, 0.f, 0.f);
        if (!same_bits(d, sep_hilo(A, Al, B, Bl).x)) ++bad_bits;
        const double exact = ((double)hb + (double)lb) - ((double)ha + (double)la);
        // the low parts' difference rounds at 2^-24 of itself, <= 2^-48 of the positions
        const double bound = ldexp(1.0, -46) * (fabs(exact) + fabs(pa) + fabs(pa + off));
        const double err = fabs(((double)d + (double)lo) - exact);
        worst = fmax(worst, err / bound);
        if (err > bound) ++bad_err;
    }
    printf("sep1_ff: bits differ %d, above the bound %d, worst error / bound %.3g\n", bad_bits, bad_err, worst);
    return bad_bits + bad_err;
}

static int check_wrap() {
    int bad_bits = 0, bad_err = 0, wrapped = 0;
    double worst = 0.0;
    const double boxes[2] = {1.0, 3.7};
    for (int t = 0; t < 200000; ++t) {
        const double box = boxes[t & 1];
        float bh, bl;
        split(box, bh, bl);
        const double boxd = (double)bh + (double)bl;
        // near the faces half of the time, so that the nearest image wraps
        const double pa = (t & 2) ? urange(0.0, 1e-3) * boxd : urange(0.0, boxd);
        const double pb = (t & 2) ? boxd - urange(1e-9, 1e-3) * boxd : urange(0.0, boxd);
        float ha, la, hb, lb;
        split(pa, ha, la);
        split(pb, hb, lb);
        float lo;
        const float r = wrap1_ff(hb, ha, lb, la, bh, bl, lo);
        if (!same_bits(r, wrap1(hb, ha, lb, la, bh, bl))) ++bad_bits;
        double exact = ((double)hb + (double)lb) - ((double)ha + (double)la);
        if (fabs((double)hb - (double)ha + (double)lb - (double)la) > 0.5 * bh) {
            exact -= copysign(boxd, exact);
            ++wrapped;
        }
        const double bound = ldexp(1.0, -46) * (fabs(exact) + fabs(pa) + fabs(pb) + boxd);
        const double err = fabs(((double)r + (double)lo) - exact);
        worst = fmax(worst, err / bound);
        if (err > bound) ++bad_err;
    }
    printf("wrap1_ff: %d wrapped, bits differ %d, above the bound %d, worst error / bound %.3g\n", wrapped,
           bad_bits, bad_err, worst);
    return bad_bits + bad_err + (wrapped < 50000);
}

static int check_scale() {
    int bad = 0;
    double worst = 0.0;
    for (int t = 0; t < 200000; ++t) {
        const double sep = urange(-1.0, 1.0) * pow(10.0, urange(-6.0, 0.0));
        float d, dlo;
        split(sep, d, dlo);
        const float hinv = (float)urange(1.0, 1e4);
        const float x = d * hinv;
        const float xl = scaled_sep_lo(d, dlo, hinv, x);
        const double exact = ((double)d + (double)dlo) * (double)hinv;
        const double err = fabs(((double)x + (double)xl) - exact) / fabs(exact);
        worst = fmax(worst, err);
        if (err > ldexp(1.0, -44)) ++bad;
    }
    printf("scaled_sep_lo: error above 2^-44 %d, worst %.3g\n", bad, worst);
    return bad;
}

// The residual of a smooth field: f_j - f_i is dominated by the linear
// prediction, the quadratic part is small and the fit residual smaller still.
static int check_residual() {
    int bad = 0;
    double worst = 0.0;
    const double u = ldexp(1.0, -24);
    for (int t = 0; t < 200000; ++t) {
        float x[3], xl[3], a[9], sol[9];
        double xe[3];
        for (int d = 0; d < 3; ++d) {
            const double v = urange(-1.0, 1.0);
            x[d] = (float)v;
            xl[d] = (float)(v - (double)x[d]);
            xe[d] = (double)x[d] + (double)xl[d];
        }
        a[0] = x[0]; a[1] = x[1]; a[2] = x[2];
        a[3] = 0.5f * x[0] * x[0]; a[4] = 0.5f * x[1] * x[1]; a[5] = 0.5f * x[2] * x[2];
        a[6] = x[0] * x[1]; a[7] = x[1] * x[2]; a[8] = x[2] * x[0];
        const double scale2 = pow(10.0, urange(-5.0, -1.0));  // second-derivative part against the first
        for (int m = 0; m < 3; ++m) sol[m] = (float)urange(-1.0, 1.0);
        for (int m = 3; m < 9; ++m) sol[m] = (float)(scale2 * urange(-1.0, 1.0));
        double lin = 0.0, quad = 0.0, qabs = 0.0;
        for (int d = 0; d < 3; ++d) lin += xe[d] * (double)sol[d];
        for (int m = 3; m < 9; ++m) {
            quad += (double)a[m] * (double)sol[m];
            qabs += fabs((double)a[m] * (double)sol[m]);
        }
        const double resid = scale2 * 1e-2 * urange(-1.0, 1.0);
        const double f0 = urange(-3.0, 3.0);
        const double fj = f0 + lin + quad + resid;
        float fh, fl, f0h, f0l;
        split(fj, fh, fl);
        split(f0, f0h, f0l);
        const float e = refine_residual<3, 9>(x, xl, a, sol, fh, fl, f0h, f0l);
        const double dfe = ((double)fh + (double)fl) - ((double)f0h + (double)f0l);
        const double eref = dfe - lin - quad;
        // FP32 rounding of the small terms (the quadratic part's FMA chain at
        // 2^-24 of its terms), float-float rounding of the large ones
        const double bound = 4.0 * u * (fabs(eref) + qabs) + 16.0 * u * u * (fabs(lin) + fabs(fj) + fabs(f0));
        const double err = fabs((double)e - eref);
        worst = fmax(worst, err / bound);
        if (err > bound) ++bad;
    }
    printf("refine_residual: above the bound %d, worst error / bound %.3g\n", bad, worst);
    return bad;
}

int main() {
    const int fails = check_sep() + check_wrap() + check_scale() + check_residual();
    printf(fails ? "FAILED %d\n" : "ok\n", fails);
    return fails ? 1 : 0;
}
