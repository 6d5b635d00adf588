// Device-wide exclusive prefix sum of uint32 (three phases: tile sums, a
// single-block scan of the tile sums with a running carry, tile scans).
#pragma once
#include "mg_common.cuh"

namespace mg {
namespace {  // internal linkage: each translation unit gets its own copy

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

inline size_t scan_workspace_bytes(int64_t n) {
    int64_t tiles = (n + kScanTile - 1) / kScanTile;
    return sizeof(uint32_t) * (size_t)(tiles + 1);
}

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *total) {
    __shared__ uint32_t wsum[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        wsum[lane] = s;
    }
    __syncthreads();
    uint32_t before = (warp > 0 ? wsum[warp - 1] : 0u) + x - v;
    *total = wsum[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before;
}

__global__ __launch_bounds__(kScanThreads) void k_scan_tiles(const uint32_t *__restrict__ in,
                                                             int64_t n, uint32_t *__restrict__ sums) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j)
        if (base + j < n) s += in[base + j];
    uint32_t tot;
    block_excl_scan(s, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ __launch_bounds__(kScanThreads) void k_scan_sums(uint32_t *__restrict__ sums, int64_t tiles) {
    uint32_t carry = 0;
    for (int64_t b = 0; b < tiles; b += kScanThreads) {
        int64_t i = b + threadIdx.x;
        uint32_t v = i < tiles ? sums[i] : 0u;
        uint32_t tot;
        uint32_t ex = block_excl_scan(v, &tot);
        if (i < tiles) sums[i] = carry + ex;
        carry += tot;
    }
}

__global__ __launch_bounds__(kScanThreads) void k_scan_apply(const uint32_t *in, uint32_t *out,
                                                             int64_t n,
                                                             const uint32_t *__restrict__ sums) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        v[j] = base + j < n ? in[base + j] : 0u;
        s += v[j];
    }
    uint32_t tot;
    uint32_t ex = block_excl_scan(s, &tot) + sums[blockIdx.x];
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        if (base + j < n) out[base + j] = ex;
        ex += v[j];
    }
}

// out may alias in.
inline int exclusive_scan_u32(const uint32_t *in, uint32_t *out, int64_t n, void *ws,
                              cudaStream_t st) {
    if (n <= 0) return MG_OK;
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    uint32_t *sums = static_cast<uint32_t *>(ws);
    k_scan_tiles<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, n, sums);
    MG_CHECK_LAUNCH();
    k_scan_sums<<<1, kScanThreads, 0, st>>>(sums, tiles);
    MG_CHECK_LAUNCH();
    k_scan_apply<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, out, n, sums);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

}  // namespace
}  // namespace mg
