// Shared device helpers for the meshoid_gb300 kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/meshoid_gb300.h"

namespace mg {

constexpr int kKeyBits = 21;                 // Morton bits per dimension
constexpr int kMaxLevel = 18;                // finest level kept contiguous by the sort
constexpr int kSortLowBit = 3 * (kKeyBits - kMaxLevel);  // 9: key bits below this are not sorted
constexpr int kWarp = 32;

// Every kernel launch of the library is followed by MG_CHECK_LAUNCH, which
// also counts it (mg_launch_count reports the total).
void count_launch();

#define MG_CHECK_LAUNCH()                                    \
    do {                                                     \
        ::mg::count_launch();                                \
        cudaError_t e_ = cudaGetLastError();                 \
        if (e_ != cudaSuccess) return MG_ERR_CUDA;           \
    } while (0)

#define MG_CUDA(call)                                        \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return MG_ERR_CUDA;           \
    } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Stable LSD radix sort (8-bit digits) of (key, value) pairs by key bits
// [bit0, bit0 + nbits), in place (csrc/mg_index.cu).
size_t radix_sort_workspace_bytes(int64_t n);
int radix_sort_pairs(uint64_t *keys, int32_t *vals, int64_t n, int bit0, int nbits, void *ws, size_t wsb,
                     cudaStream_t st);

inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// Bump allocator over a caller workspace.
struct Carve {
    char *base;
    size_t cap, used;
    Carve(void *p, size_t c) : base(static_cast<char *>(p)), cap(c), used(0) {}
    template <class T>
    T *take(size_t count) {
        size_t off = align_up(used);
        used = off + count * sizeof(T);
        return used <= cap ? reinterpret_cast<T *>(base + off) : nullptr;
    }
    bool ok() const { return used <= cap; }
};

// Cubic spline, un-normalised: src/meshoid/kernel_density.py:82-96.  Both
// pieces are evaluated and one is selected (no divergent branch when the lanes
// of a warp hold different q); for q > 1 the outer piece is 0 because
// a = max(1 - q, 0).
__host__ __device__ __forceinline__ float spline_w(float q) {
    const float inner = fmaf(q * q, fmaf(6.0f, q, -6.0f), 1.0f);
    const float a = fmaxf(1.0f - q, 0.0f);
    const float outer = 2.0f * a * a * a;
    return q <= 0.5f ? inner : outer;
}

// The reference's truncations of y0 = (x - h) / dx + 1 and y1 = (x + h) / dx
// (C conversion toward zero of the FP64 quotients, grid_deposition.py
// footprints), decided in FP32 from the FP32 roundings of x, h and 1 / dx
// where that can tell: each FP32 value lies within ~4e-7 (|x| + h) / dx of the
// FP64 one, so where both lie farther than 1e-6 (|x| + h) / dx + 1e-6 from an
// integer they truncate alike.  Returns false (the caller decides in FP64)
// otherwise, which includes every |y| beyond 2^23 and NaN.
__host__ __device__ __forceinline__ bool trunc_pair32(float x, float h, float inv_dx, int &a, int &b) {
    const float y0 = (x - h) * inv_dx + 1.0f, y1 = (x + h) * inv_dx;
    const float m = 1e-6f * (fabsf(x) + h) * inv_dx + 1e-6f;
    if (!(fabsf(y0 - rintf(y0)) > m && fabsf(y1 - rintf(y1)) > m)) return false;
    a = (int)y0;
    b = (int)y1;
    return true;
}

// Half the spline above, w(q) / 2, by the same operations scaled by 1/2:
// every rounding step scales exactly (no intermediate is subnormal for
// 0 <= q), so spline_w_half(q) == spline_w(q) / 2 for every float q, and
// (w / 2) * (2 c) equals w * c bit for bit; the factor 2 of the outer branch
// moves into the caller's coefficient.
__host__ __device__ __forceinline__ float spline_w_half(float q) {
    const float inner = fmaf(q * q, fmaf(3.0f, q, -3.0f), 0.5f);
    const float a = fmaxf(1.0f - q, 0.0f);
    const float outer = a * a * a;
    return q <= 0.5f ? inner : outer;
}

// d W / d q of the spline above.
__host__ __device__ __forceinline__ float spline_dw(float q) {
    const float inner = q * fmaf(18.0f, q, -12.0f);
    const float a = fmaxf(1.0f - q, 0.0f);
    const float outer = -6.0f * a * a;
    return q <= 0.5f ? inner : outer;
}

// Spread the low 21 bits of v so bit i lands at bit 3i.
__host__ __device__ __forceinline__ uint64_t spread3(uint64_t v) {
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

__host__ __device__ __forceinline__ uint64_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}

// ---- cell lookup ---------------------------------------------------------------
constexpr int kBrickWords = MG_BRICK_WORDS;
constexpr int kBrickChild = 513;  // offset of the child table in a brick
constexpr int kBrickRange = 1025; // offset of the brick's [begin, end) slot range

__device__ __forceinline__ uint32_t lower_bound_prefix(const uint64_t *__restrict__ keys, uint32_t a,
                                                       uint32_t b, uint64_t code, int ks) {
    while (a < b) {
        uint32_t m = a + ((b - a) >> 1);
        if ((keys[m] >> ks) < code)
            a = m + 1;
        else
            b = m;
    }
    return a;
}

struct CellIndex {
    int Lg;
    const uint64_t *keys;
    const uint32_t *cs;
    const int32_t *brick_of;  // may be null
    const uint32_t *bricks;
};

// Slot range [a, b) of the level-L cell with Morton code `code`: dense table
// for L <= Lg; below it, descend the bricks (one dependent lookup per three
// levels) and binary-search the keys only inside a cell without a brick.
__device__ __forceinline__ void cell_lookup(const CellIndex &ci, int L, uint64_t code, uint32_t &a, uint32_t &b) {
    if (L <= ci.Lg) {
        const int sh = 3 * (ci.Lg - L);
        a = __ldg(ci.cs + (code << sh));
        b = __ldg(ci.cs + ((code + 1) << sh));
        return;
    }
    const uint64_t c = code >> (3 * (L - ci.Lg));
    uint32_t A = __ldg(ci.cs + c), B = __ldg(ci.cs + c + 1);
    int br = ci.brick_of ? __ldg(ci.brick_of + c) : -1;
    int base = ci.Lg;
    while (br >= 0) {
        const uint32_t *st = ci.bricks + (size_t)br * kBrickWords;
        if (L <= base + 3) {
            const int shift = 3 * (base + 3 - L);
            const uint32_t local = (uint32_t)(code & ((1ull << (3 * (L - base))) - 1ull));
            a = __ldg(st + (local << shift));
            b = __ldg(st + ((local + 1) << shift));
            return;
        }
        const uint32_t sub = (uint32_t)((code >> (3 * (L - base - 3))) & 511ull);
        A = __ldg(st + sub);
        B = __ldg(st + sub + 1);
        br = (int)__ldg(st + kBrickChild + sub);
        base += 3;
    }
    const int ks = 3 * (kKeyBits - L);
    a = lower_bound_prefix(ci.keys, A, B, code, ks);
    b = lower_bound_prefix(ci.keys, a, B, code + 1, ks);
}

// Frame layout in device memory (8 doubles).
struct Frame {
    double ox, oy, oz, side, inv_side, cx, cy, cz;
};

__device__ __forceinline__ Frame load_frame(const double *f) {
    Frame r;
    r.ox = f[0]; r.oy = f[1]; r.oz = f[2]; r.side = f[3];
    r.inv_side = f[4]; r.cx = f[5]; r.cy = f[6]; r.cz = f[7];
    return r;
}

// FP32 separation from slot a to slot b using the hi/lo split: the hi parts of
// nearby particles differ exactly or to half an ulp of the difference, so the
// result carries ~24 significant bits of the true separation.
__host__ __device__ __forceinline__ float3 sep_hilo(float4 ha, float4 la, float4 hb, float4 lb) {
    return make_float3((hb.x - ha.x) + (lb.x - la.x), (hb.y - ha.y) + (lb.y - la.y),
                       (hb.z - ha.z) + (lb.z - la.z));
}

// Error-free FP32 sum (Knuth TwoSum): s + e == a + b exactly.
__host__ __device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Nearest-image separation component (src/meshoid/derivatives.py:9-15) from
// the hi/lo split.  A wrapped separation is much smaller than the operands, so
// both subtractions are carried error-free (TwoSum) and the box is an FP32
// pair box_hi + box_lo.
__host__ __device__ __forceinline__ float wrap1(float hb, float ha, float lb, float la, float box_hi, float box_lo) {
    float s, e;
    two_sum(hb, -ha, s, e);
    const float l = lb - la;
    const float d = s + (e + l);
    if (fabsf(d) > 0.5f * box_hi) {
        const float sg = d > 0.0f ? 1.0f : -1.0f;
        float s2, e2;
        two_sum(s, -sg * box_hi, s2, e2);
        return s2 + ((e2 + e + l) - sg * box_lo);
    }
    return d;
}

__host__ __device__ __forceinline__ float3 sep_hilo_periodic(float4 ha, float4 la, float4 hb, float4 lb,
                                                    float box_hi, float box_lo) {
    return make_float3(wrap1(hb.x, ha.x, lb.x, la.x, box_hi, box_lo), wrap1(hb.y, ha.y, lb.y, la.y, box_hi, box_lo),
                       wrap1(hb.z, ha.z, lb.z, la.z, box_hi, box_lo));
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

}  // namespace mg
