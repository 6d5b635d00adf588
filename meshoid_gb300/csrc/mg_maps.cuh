// Map tile helpers shared by the kernels of mg_maps.cu and the host check
// tests/native/sd_cull_check.cu.
#pragma once
#include <math.h>

namespace mg {

// k_sd_tile_pairs: true when a 16 x 8 sub-block of pixel nodes (origin bx0,
// by0 as exact small floats) can skip the record (pa = rx, ry, 1/h, coef;
// pb = gx0, gx1 - gx0, gy0, gy1 - gy0 as exact small floats): its nodes miss
// the footprint box, or the nearest of them lies beyond h by more than 1e-4
// of h^2, so that every node evaluates q > 1 and weighs exactly 0.  The
// nearest node's offsets are the ones the pixels form (ddx = rx - (gx - gx0)
// dx by one fmaf, monotonic in gx), so the test bounds the pixels' own
// FP32 values.
__host__ __device__ __forceinline__ bool sd_block_skips(float bx0, float by0, float4 pa, float4 pb, float dxf) {
    const float ox0 = bx0 - pb.x, oy0 = by0 - pb.z;
    if (ox0 + 15.0f < 0.0f || ox0 > pb.y || oy0 + 7.0f < 0.0f || oy0 > pb.w) return true;
    const float ex = fmaxf(0.0f, fmaxf(fmaf(-(ox0 + 15.0f), dxf, pa.x), -fmaf(-ox0, dxf, pa.x)));
    const float ey = fmaxf(0.0f, fmaxf(fmaf(-(oy0 + 7.0f), dxf, pa.y), -fmaf(-oy0, dxf, pa.y)));
    return fmaf(ex, ex, ey * ey) * (pa.z * pa.z) > 1.0001f;
}

}  // namespace mg
