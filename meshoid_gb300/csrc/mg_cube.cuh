// Flat node index -> (i, j, l) of a particle's node cube, shared by the 3-D
// deposits (mg_deposit.cu).  Host and device: the CPU tests build this header
// into a host program that checks the float-reciprocal path against integer
// division.
#pragma once
#include <stdint.h>

namespace mg {

// Node (i, j, l) of a cube of ny * nz columns from a flat index.  Below 2^22
// nodes the quotients come from float reciprocals: (c + 0.5) / nz lies at
// least 0.5 / nz from an integer, and the product's relative error (2^-23)
// stays below that while c + 0.5 < 2^22.  This avoids emulated 64-bit
// division; larger cubes divide exactly.
struct CubeDiv {
    int ny, nz;
    float inv_ny, inv_nz;
    bool small;
};

__host__ __device__ __forceinline__ CubeDiv cube_div(int ny, int nz, int64_t total) {
    CubeDiv d;
    d.ny = ny;
    d.nz = nz;
    d.inv_ny = 1.0f / (float)ny;
    d.inv_nz = 1.0f / (float)nz;
    d.small = total < (1ll << 22);
    return d;
}

__host__ __device__ __forceinline__ void cube_node(int64_t c, const CubeDiv &d, int &i, int &j, int &l) {
    if (d.small) {
        const int ci = (int)c;
        const int col = (int)(((float)ci + 0.5f) * d.inv_nz);
        l = ci - col * d.nz;
        i = (int)(((float)col + 0.5f) * d.inv_ny);
        j = col - i * d.ny;
        return;
    }
    const int64_t col = c / d.nz;
    l = (int)(c - col * d.nz);
    i = (int)(col / d.ny);
    j = (int)(col - (int64_t)i * d.ny);
}

}  // namespace mg
