// Host check of trunc_pair32 (meshoid_gb300/csrc/mg_common.cuh), the FP32
// decision behind the column maps' footprints (sd_bounds32, mg_maps.cu) and
// the 3-D deposits' node ranges (gd_range, mg_deposit.cu): whenever it
// decides, both truncations must equal the reference's FP64 ones,
// (int)((x - h) / dx + 1) and (int)((x + h) / dx) (grid_deposition.py
// footprints), on random footprints across 60 binades of dx, on footprints
// placed within 1e-12 .. 1e-1 of an integer boundary, and on footprints far
// from the map's origin.  Prints "ok" on success.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>

#include "mg_common.cuh"

int main() {
    std::mt19937_64 rng(17);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    long cases = 0, decided = 0, wrong = 0;
    auto check = [&](double xs, double hs, double dx) {
        if (!(hs > 0.0) || !(dx > 0.0)) return;
        ++cases;
        int a = 0, b = 0;
        if (!mg::trunc_pair32((float)xs, (float)hs, (float)(1.0 / dx), a, b)) return;
        ++decided;
        const int a64 = (int)((xs - hs) / dx + 1), b64 = (int)((xs + hs) / dx);
        if (a != a64 || b != b64) {
            if (wrong < 5)
                std::printf("  x %.17g h %.17g dx %.17g: FP32 %d %d, FP64 %d %d\n", xs, hs, dx, a, b, a64, b64);
            ++wrong;
        }
    };
    for (int i = 0; i < 3000000; ++i) {
        const double dx = std::ldexp(1.0 + u(rng), (int)(u(rng) * 60) - 30);
        const double hs = dx * std::ldexp(1.0 + u(rng), (int)(u(rng) * 24) - 12);
        const int mode = i % 4;
        double xs;
        if (mode == 0) {
            xs = dx * (u(rng) * 5000.0 - 2000.0);
        } else if (mode == 3) {
            xs = dx * std::ldexp(1.0 + u(rng), 10 + (int)(u(rng) * 20)) * (u(rng) < 0.5 ? -1.0 : 1.0);
        } else {
            // an end of the footprint within delta of a node: y0 = n + delta or y1 = n + delta
            const double n = std::floor(u(rng) * 5100.0) - 100.0;
            const double delta = (u(rng) < 0.1 ? 0.0 : std::pow(10.0, -1.0 - 11.0 * u(rng))) * (u(rng) < 0.5 ? -1.0 : 1.0);
            xs = mode == 1 ? (n - 1.0 + delta) * dx + hs : (n + delta) * dx - hs;
        }
        check(xs, hs, dx);
    }
    std::printf("trunc_pair32: %ld footprints, %ld decided in FP32 (%.1f%%), %ld differ from the FP64 truncations\n",
                cases, decided, 100.0 * decided / (double)cases, wrong);
    if (wrong != 0 || decided == 0) return 1;
    std::printf("ok\n");
    return 0;
}
