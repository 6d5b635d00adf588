// Host check of the large-footprint map kernel's two exactness arguments
// (k_sd_tile_pairs, meshoid_gb300/csrc/mg_maps.cu), with the kernel's FP32
// arithmetic restated and its rsqrtf modelled as the correctly rounded
// 1 / sqrt times (1 + e), |e| <= 2^-21:
//  * sd_block_skips (mg_maps.cuh): whenever it lets a 16 x 8 sub-block skip a
//    record, every node of the sub-block evaluates q > 1, a weight of exactly
//    0, so the skip changes no pixel;
//  * no per-pixel box test: a node outside the footprint box (the reference's
//    FP64 truncations) weighs at most 1e-18 of the peak weight (the rsqrtf
//    error bounds 1 - q by ~5e-7 there; 1.1e-20 was the largest seen).
// Footprints as k_sd_prep forms them: x and h in FP64, gx0 = trunc((x - h) /
// dx + 1), gx1 = trunc((x + h) / dx) clamped to the map, rx = x - gx0 dx in
// FP32.  Prints "ok" on success.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>

#include <cuda_runtime.h>

#include "mg_common.cuh"
#include "mg_maps.cuh"

static float q_of(float ddx, float ddy, float hinv, float e) {
    const float r2 = std::fmaf(ddx, ddx, ddy * ddy);
    const float rs = (1.0f / std::sqrt(std::fmax(r2, 1e-30f))) * (1.0f + e);
    return (r2 * rs) * hinv;
}

int main() {
    std::mt19937_64 rng(5);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    const int res = 1024;
    const float eps[3] = {-std::ldexp(1.0f, -21), 0.0f, std::ldexp(1.0f, -21)};
    long cases = 0, skipped = 0, circle_skips = 0, bad_skip = 0, outside = 0;
    double worst_outside = 0.0;
    for (int it = 0; it < 400000; ++it) {
        const double size = std::ldexp(1.0, (int)(u(rng) * 40) - 20);  // map side 2^-20 .. 2^20
        const double dx = size / res;
        const double x = u(rng) * size, y = u(rng) * size;
        const double h = dx * std::exp(u(rng) * std::log(200.0)) * 0.5;  // 0.5 .. 100 pixels
        int gx0 = std::max((int)((x - h) / dx + 1.0), 0), gx1 = std::min((int)((x + h) / dx), res - 1);
        int gy0 = std::max((int)((y - h) / dx + 1.0), 0), gy1 = std::min((int)((y + h) / dx), res - 1);
        if (gx0 > gx1 || gy0 > gy1) continue;
        const float dxf = (float)dx, hinv = 1.0f / (float)h;
        const float4 pa = make_float4((float)(x - gx0 * dx), (float)(y - gy0 * dx), hinv, 1.0f);
        const float4 pb = make_float4((float)gx0, (float)(gx1 - gx0), (float)gy0, (float)(gy1 - gy0));
        // sub-blocks of the tiles around the footprint (16 x 8 grid)
        for (int bx = std::max(0, gx0 / 16 - 1) * 16; bx <= std::min(res - 16, (gx1 / 16 + 1) * 16); bx += 16)
            for (int by = std::max(0, gy0 / 8 - 1) * 8; by <= std::min(res - 8, (gy1 / 8 + 1) * 8); by += 8) {
                ++cases;
                const bool box_miss = bx + 15 < gx0 || bx > gx1 || by + 7 < gy0 || by > gy1;
                if (!mg::sd_block_skips((float)bx, (float)by, pa, pb, dxf)) continue;
                ++skipped;
                if (box_miss) continue;  // nodes outside the box: checked below
                ++circle_skips;
                for (int r = 0; r < 16; ++r)
                    for (int c = 0; c < 8; ++c) {
                        const float ddx = std::fmaf(-((float)(bx + r) - pb.x), dxf, pa.x);
                        const float ddy = std::fmaf(-((float)(by + c) - pb.z), dxf, pa.y);
                        for (float e : eps)
                            if (!(q_of(ddx, ddy, hinv, e) > 1.0f)) ++bad_skip;
                    }
            }
        // nodes just outside the footprint box, along its four edges
        for (int t = -1; t <= (gy1 - gy0) + 1; ++t)
            for (int side = 0; side < 2; ++side) {
                const int gx = side ? gx1 + 1 : gx0 - 1, gy = gy0 + t;
                if (gx < 0 || gx >= res || gy < 0 || gy >= res) continue;
                const float ddx = std::fmaf(-((float)gx - pb.x), dxf, pa.x);
                const float ddy = std::fmaf(-((float)gy - pb.z), dxf, pa.y);
                for (float e : eps) {
                    worst_outside = std::fmax(worst_outside, mg::spline_w_half(q_of(ddx, ddy, hinv, e)) / 0.5);
                    ++outside;
                }
            }
        for (int t = 0; t <= gx1 - gx0; ++t)
            for (int side = 0; side < 2; ++side) {
                const int gy = side ? gy1 + 1 : gy0 - 1, gx = gx0 + t;
                if (gx < 0 || gx >= res || gy < 0 || gy >= res) continue;
                const float ddx = std::fmaf(-((float)gx - pb.x), dxf, pa.x);
                const float ddy = std::fmaf(-((float)gy - pb.z), dxf, pa.y);
                for (float e : eps) {
                    worst_outside = std::fmax(worst_outside, mg::spline_w_half(q_of(ddx, ddy, hinv, e)) / 0.5);
                    ++outside;
                }
            }
    }
    std::printf("sub-blocks tested %ld, skipped %ld (%ld inside the box, by the circle test), "
                "nodes of circle-skipped sub-blocks with q <= 1: %ld; %ld nodes outside footprint boxes, "
                "largest weight / peak %.3e\n",
                cases, skipped, circle_skips, bad_skip, outside, worst_outside);
    if (bad_skip != 0 || circle_skips == 0 || worst_outside > 1e-18) return 1;
    std::printf("ok\n");
    return 0;
}
