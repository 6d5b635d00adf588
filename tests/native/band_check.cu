// Host check of the warp-per-query search's FP64 re-decision band
// (meshoid_gb300/csrc/mg_knn.cu): candidates whose FP32 squared distance lies
// within kBandEps = 1e-5 (relative) of the k-th are re-ranked in FP64, so the
// FP32 squared distance of the hi/lo separations (sep_hilo, wrap1 of
// mg_common.cuh; the same FMA expression as cand_d2p) must stay well inside
// 1e-5 of the true one, in open and periodic boxes.  It does at separations
// of at least 1e-7 of the coordinates' magnitude (asserted); closer pairs
// are reported: there the hi/lo split's own rounding (2^-48 of the
// coordinates) approaches the band.  Built and run on the CPU by
// tests/test_native_helpers.py.
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include "mg_common.cuh"

using namespace mg;

static uint64_t rng_state = 0x632BE59BD9B4E019ull;
static double urand() {
    rng_state ^= rng_state >> 12;
    rng_state ^= rng_state << 25;
    rng_state ^= rng_state >> 27;
    return (double)((rng_state * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0);
}

static void split(double v, float &h, float &l) {
    h = (float)v;
    l = (float)(v - (double)h);
}

int main() {
    double worst = 0.0, worst_deep = 0.0;
    long long checked = 0;
    for (int t = 0; t < 2000000; ++t) {
        const bool periodic = t & 1;
        const double box = periodic ? pow(10.0, -2.0 + 4.0 * urand()) : 0.0;
        const double span = periodic ? box : pow(10.0, -3.0 + 6.0 * urand());
        double a[3], b[3];
        const double sep = span * pow(10.0, -9.0 * urand());
        for (int d = 0; d < 3; ++d) {
            a[d] = span * urand();
            b[d] = a[d] + sep * (2.0 * urand() - 1.0);
            if (periodic) {  // across the face half of the time
                if (t & 2) b[d] = fmod(b[d] + box, box);
                else b[d] = fmin(fmax(b[d], 0.0), box * (1 - 1e-16));
            }
        }
        float4 ha, la, hb, lb;
        split(a[0], ha.x, la.x); split(a[1], ha.y, la.y); split(a[2], ha.z, la.z);
        split(b[0], hb.x, lb.x); split(b[1], hb.y, lb.y); split(b[2], hb.z, lb.z);
        ha.w = la.w = hb.w = lb.w = 0.0f;
        float bh, bl;
        split(box, bh, bl);
        const float3 sv = periodic ? sep_hilo_periodic(ha, la, hb, lb, bh, bl) : sep_hilo(ha, la, hb, lb);
        const float d2 = fmaf(sv.z, sv.z, fmaf(sv.y, sv.y, sv.x * sv.x));
        double e2 = 0.0;
        const double bx = (double)bh + (double)bl;
        const double pa[3] = {(double)ha.x + la.x, (double)ha.y + la.y, (double)ha.z + la.z};
        const double pb[3] = {(double)hb.x + lb.x, (double)hb.y + lb.y, (double)hb.z + lb.z};
        for (int d = 0; d < 3; ++d) {
            double v = pb[d] - pa[d];
            if (periodic && fabs(v) > 0.5 * bx) v -= copysign(bx, v);
            e2 += v * v;
        }
        if (e2 == 0.0) continue;
        const double rel = fabs((double)d2 - e2) / e2;
        // the low parts' difference rounds at 2^-24 of itself, i.e. 2^-48 of
        // the coordinates: relative to the separation that grows as the
        // separation shrinks against the coordinates' magnitude
        double xm = 0.0;
        for (int d = 0; d < 3; ++d) xm = fmax(xm, fmax(fabs(pa[d]), fabs(pb[d])));
        const double ratio = sqrt(e2) / xm;
        if (ratio >= 1e-7) worst = fmax(worst, rel);
        else worst_deep = fmax(worst_deep, rel);
        ++checked;
    }
    const bool ok = worst < 0.1 * 1e-5;  // at least 10x inside the band
    printf("warp-path band: %lld separations, worst relative error of the FP32 d^2 %.3g at separations >= 1e-7 of "
           "the coordinates (band 1e-5), %.3g below that\n", checked, worst, worst_deep);
    printf(ok ? "ok\n" : "FAILED\n");
    return ok ? 0 : 1;
}
