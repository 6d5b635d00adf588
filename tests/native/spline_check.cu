// Host check of spline_w_half (meshoid_gb300/csrc/mg_common.cuh), which the
// map tile kernels use with a doubled coefficient in place of spline_w: it
// must equal spline_w(q) / 2 exactly for every float q the kernels evaluate
// (every float in [1/4, 1.0625], a stride through [0, 1/4), and q beyond 1),
// and fmaf(w / 2, 2 c, acc) must equal fmaf(w, c, acc) on random
// coefficients and partial sums.  Prints "ok" on success.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "mg_common.cuh"

static float from_bits(uint32_t b) {
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}
static uint32_t bits(float f) {
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return b;
}

int main() {
    using mg::spline_w;
    using mg::spline_w_half;
    long bad = 0, checked = 0;
    auto check_q = [&](float q) {
        const float w = spline_w(q), wh = spline_w_half(q);
        ++checked;
        if (bits(wh) != bits(0.5f * w)) {
            if (bad < 5) std::printf("q %.9g: w %.9g, half %.9g\n", q, w, wh);
            ++bad;
        }
    };
    const uint32_t b_quarter = bits(0.25f), b_end = bits(1.0625f);
    for (uint32_t b = 0; b < b_quarter; b += 97) check_q(from_bits(b));
    for (uint32_t b = b_quarter; b <= b_end; ++b) check_q(from_bits(b));
    for (float q : {1.5f, 2.0f, 17.0f, 1e30f}) check_q(q);
    std::mt19937_64 rng(11);
    std::uniform_real_distribution<float> uq(0.0f, 1.0f), um(-1.0f, 1.0f);
    std::uniform_int_distribution<int> ue(-60, 60);
    long bad_fma = 0;
    for (int i = 0; i < 2000000; ++i) {
        const float q = uq(rng);
        const float c = std::ldexp(um(rng), ue(rng)), acc = std::ldexp(um(rng), ue(rng));
        const float c2 = 2.0f * c;
        if (bits(std::fmaf(spline_w_half(q), c2, acc)) != bits(std::fmaf(spline_w(q), c, acc))) ++bad_fma;
    }
    std::printf("spline_w_half: %ld values of q checked, %ld differ; fma with doubled coefficient: %ld of 2000000 differ\n",
                checked, bad, bad_fma);
    if (bad || bad_fma) return 1;
    std::printf("ok\n");
    return 0;
}
