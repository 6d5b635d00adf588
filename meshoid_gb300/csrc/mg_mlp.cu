// Seed network: 54 -> 64 -> 64 -> 1 MLP (GELU) that predicts log(h / s) from
// cell-occupancy features (s = side of the query's adaptive cell).  Not part
// of the reference: it only supplies the first search radius and the first
// h guess; the converged neighbours and h are those of the plain solve.
//
// Inference (mg_mlp_forward): tensor cores, mma.sync m16n8k16 bf16 x bf16 ->
// f32, one warp per 16-row tile, weights staged in shared memory.  The hidden
// activations go from the f32 accumulator fragments straight into the bf16 A
// fragments of the next layer (the m16n8 C layout of two adjacent n-tiles is
// the m16k16 A layout).
//
// Training (mg_mlp_train_step): FP32 SIMT forward + backward over a batch
// tile in shared memory (the forward rounds weights and inputs to bf16 exactly
// as inference sees them), per-block gradient partials reduced with atomics,
// then an Adam update of the FP32 master weights and a refresh of the bf16
// copies.
#include <cuda_bf16.h>

#include "mg_common.cuh"

namespace mg {

constexpr int kIn = MG_MLP_IN_PAD;  // 64 (54 used)
constexpr int kHid = MG_MLP_HIDDEN; // 64
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kHid * kIn;
constexpr int kOffW2 = kOffB1 + kHid;
constexpr int kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid;
constexpr int kOffB3 = kOffW3 + kHid;
static_assert(kOffB3 + 1 == MG_MLP_PARAM_COUNT, "parameter layout");

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.3989422804014327f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x = lo (low half)
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ---- inference -------------------------------------------------------------------
__global__ __launch_bounds__(128) void k_mlp_forward(const uint16_t *__restrict__ feat, int64_t n,
                                                     const uint16_t *__restrict__ w1, const float *__restrict__ b1,
                                                     const uint16_t *__restrict__ w2, const float *__restrict__ b2,
                                                     const uint16_t *__restrict__ w3, const float *__restrict__ b3,
                                                     const float *__restrict__ cell_side, float *__restrict__ out,
                                                     float *__restrict__ seed_h) {
    __shared__ uint32_t s_w1[kHid * kIn / 2], s_w2[kHid * kHid / 2];
    __shared__ float s_b1[kHid], s_b2[kHid], s_w3[kHid];
    const uint32_t *gw1 = reinterpret_cast<const uint32_t *>(w1);
    const uint32_t *gw2 = reinterpret_cast<const uint32_t *>(w2);
    for (int i = threadIdx.x; i < kHid * kIn / 2; i += blockDim.x) {
        s_w1[i] = gw1[i];
        s_w2[i] = gw2[i];
    }
    for (int i = threadIdx.x; i < kHid; i += blockDim.x) {
        s_b1[i] = b1[i];
        s_b2[i] = b2[i];
        s_w3[i] = __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(w3 + i));
    }
    __syncthreads();
    const float bias3 = b3[0];
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int64_t ntile = (n + 15) / 16;
    const int64_t warp0 = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    const int64_t nwarp = (int64_t)gridDim.x * (blockDim.x >> 5);
    const uint32_t *x32 = reinterpret_cast<const uint32_t *>(feat);
    for (int64_t tile = warp0; tile < ntile; tile += nwarp) {
        const int64_t r0 = tile * 16 + g, r1 = r0 + 8;
        // A fragments of the input tile: 4 k-steps of 16 features
        uint32_t a[4][4];
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            const int col = ks * 16 + 2 * t;  // bf16 index; /2 -> uint32 index
            a[ks][0] = r0 < n ? x32[(r0 * kIn + col) / 2] : 0u;
            a[ks][1] = r1 < n ? x32[(r1 * kIn + col) / 2] : 0u;
            a[ks][2] = r0 < n ? x32[(r0 * kIn + col + 8) / 2] : 0u;
            a[ks][3] = r1 < n ? x32[(r1 * kIn + col + 8) / 2] : 0u;
        }
        // layer 1
        float c1[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            c1[nt][0] = c1[nt][1] = c1[nt][2] = c1[nt][3] = 0.0f;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                const int nrow = nt * 8 + g;  // output unit (B column)
                const uint32_t b0 = s_w1[(nrow * kIn + ks * 16 + 2 * t) / 2];
                const uint32_t bb1 = s_w1[(nrow * kIn + ks * 16 + 2 * t + 8) / 2];
                mma_bf16(c1[nt], a[ks], b0, bb1);
            }
        }
        // bias + GELU -> bf16 A fragments of layer 2
        uint32_t a2[4][4];
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                const int nt = 2 * ks + half;
                const int u = nt * 8 + 2 * t;
                const float v0 = gelu(c1[nt][0] + s_b1[u]), v1 = gelu(c1[nt][1] + s_b1[u + 1]);
                const float v2 = gelu(c1[nt][2] + s_b1[u]), v3 = gelu(c1[nt][3] + s_b1[u + 1]);
                a2[ks][half * 2 + 0] = pack_bf16(v0, v1);
                a2[ks][half * 2 + 1] = pack_bf16(v2, v3);
            }
        }
        // layer 2 + layer 3 (dot with w3) fused
        float part0 = 0.0f, part1 = 0.0f;
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                const int nrow = nt * 8 + g;
                const uint32_t b0 = s_w2[(nrow * kHid + ks * 16 + 2 * t) / 2];
                const uint32_t bb1 = s_w2[(nrow * kHid + ks * 16 + 2 * t + 8) / 2];
                const uint32_t af[4] = {a2[ks][0], a2[ks][1], a2[ks][2], a2[ks][3]};
                mma_bf16(c, af, b0, bb1);
            }
            const int u = nt * 8 + 2 * t;
            const float h0 = bf16r(gelu(c[0] + s_b2[u])), h1 = bf16r(gelu(c[1] + s_b2[u + 1]));
            const float h2 = bf16r(gelu(c[2] + s_b2[u])), h3 = bf16r(gelu(c[3] + s_b2[u + 1]));
            part0 += h0 * s_w3[u] + h1 * s_w3[u + 1];
            part1 += h2 * s_w3[u] + h3 * s_w3[u + 1];
        }
        part0 += __shfl_xor_sync(0xffffffffu, part0, 1);
        part0 += __shfl_xor_sync(0xffffffffu, part0, 2);
        part1 += __shfl_xor_sync(0xffffffffu, part1, 1);
        part1 += __shfl_xor_sync(0xffffffffu, part1, 2);
        if (t == 0) {
            // the seed h is kept within 2^+-6 of the adaptive cell side
            if (r0 < n) {
                const float o = part0 + bias3;
                out[r0] = o;
                if (seed_h) seed_h[r0] = expf(fminf(fmaxf(o, -4.2f), 4.2f)) * cell_side[r0];
            }
            if (r1 < n) {
                const float o = part1 + bias3;
                out[r1] = o;
                if (seed_h) seed_h[r1] = expf(fminf(fmaxf(o, -4.2f), 4.2f)) * cell_side[r1];
            }
        }
    }
}

// ---- training --------------------------------------------------------------------
constexpr int kTrainRows = 64;  // rows per block tile

struct TrainSmem {
    float x[kTrainRows][kIn];
    float z1[kTrainRows][kHid];
    float z2[kTrainRows][kHid];
    float dz[kTrainRows][kHid];  // dZ2, then dZ1
    float w1[kHid][kIn + 1];
    float w2[kHid][kHid + 1];
    float b1[kHid], b2[kHid], w3[kHid];
    float dout[kTrainRows];
};

__global__ __launch_bounds__(256) void k_mlp_train(const uint16_t *__restrict__ feat, const float *__restrict__ target,
                                                   int64_t n, const float *__restrict__ params,
                                                   float *__restrict__ grads, float *__restrict__ loss_sum) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem &S = *reinterpret_cast<TrainSmem *>(smem_raw);
    const int tid = threadIdx.x, nth = blockDim.x;
    // weights as inference sees them (bf16-rounded), biases FP32
    for (int i = tid; i < kHid * kIn; i += nth) S.w1[i / kIn][i % kIn] = bf16r(params[kOffW1 + i]);
    for (int i = tid; i < kHid * kHid; i += nth) S.w2[i / kHid][i % kHid] = bf16r(params[kOffW2 + i]);
    for (int i = tid; i < kHid; i += nth) {
        S.b1[i] = params[kOffB1 + i];
        S.b2[i] = params[kOffB2 + i];
        S.w3[i] = bf16r(params[kOffW3 + i]);
    }
    const float b3 = params[kOffB3];
    const int64_t r0 = (int64_t)blockIdx.x * kTrainRows;
    for (int i = tid; i < kTrainRows * kIn; i += nth) {
        const int r = i / kIn, c = i % kIn;
        const int64_t row = r0 + r;
        float v = 0.0f;
        if (row < n) v = __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(feat + row * kIn + c));
        S.x[r][c] = v;
    }
    __syncthreads();
    // layer 1: z1 = W1 x + b1
    for (int i = tid; i < kTrainRows * kHid; i += nth) {
        const int r = i / kHid, u = i % kHid;
        float s = S.b1[u];
        for (int c = 0; c < kIn; ++c) s += S.w1[u][c] * S.x[r][c];
        S.z1[r][u] = s;
    }
    __syncthreads();
    // layer 2: z2 = W2 bf16(gelu(z1)) + b2
    for (int i = tid; i < kTrainRows * kHid; i += nth) {
        const int r = i / kHid, u = i % kHid;
        float s = S.b2[u];
        for (int v = 0; v < kHid; ++v) s += S.w2[u][v] * bf16r(gelu(S.z1[r][v]));
        S.z2[r][u] = s;
    }
    __syncthreads();
    // output and loss gradient: out = w3 . bf16(gelu(z2)) + b3, loss = mean (out - t)^2
    const float inv_n = 1.0f / (float)n;
    if (tid < kTrainRows) {
        const int64_t row = r0 + tid;
        float o = b3;
        for (int u = 0; u < kHid; ++u) o += S.w3[u] * bf16r(gelu(S.z2[tid][u]));
        float d = 0.0f;
        if (row < n) {
            const float e = o - target[row];
            d = 2.0f * e * inv_n;
            atomicAdd(loss_sum, e * e * inv_n);
        }
        S.dout[tid] = d;
    }
    __syncthreads();
    // dW3, db3
    if (tid < kHid) {
        float s = 0.0f;
        for (int r = 0; r < kTrainRows; ++r) s += S.dout[r] * bf16r(gelu(S.z2[r][tid]));
        atomicAdd(&grads[kOffW3 + tid], s);
    }
    if (tid == kHid) {
        float s = 0.0f;
        for (int r = 0; r < kTrainRows; ++r) s += S.dout[r];
        atomicAdd(&grads[kOffB3], s);
    }
    // dZ2 = dout * w3 * gelu'(z2)
    for (int i = tid; i < kTrainRows * kHid; i += nth) {
        const int r = i / kHid, u = i % kHid;
        S.dz[r][u] = S.dout[r] * S.w3[u] * gelu_grad(S.z2[r][u]);
    }
    __syncthreads();
    // dW2[u][v] = sum_r dZ2[r][u] * h1[r][v];  db2[u] = sum_r dZ2[r][u]
    for (int i = tid; i < kHid * kHid; i += nth) {
        const int u = i / kHid, v = i % kHid;
        float s = 0.0f;
        for (int r = 0; r < kTrainRows; ++r) s += S.dz[r][u] * bf16r(gelu(S.z1[r][v]));
        atomicAdd(&grads[kOffW2 + i], s);
    }
    if (tid < kHid) {
        float s = 0.0f;
        for (int r = 0; r < kTrainRows; ++r) s += S.dz[r][tid];
        atomicAdd(&grads[kOffB2 + tid], s);
    }
    __syncthreads();
    // dZ1[r][v] = (sum_u dZ2[r][u] W2[u][v]) * gelu'(z1[r][v]); reuse z2 storage for it
    for (int i = tid; i < kTrainRows * kHid; i += nth) {
        const int r = i / kHid, v = i % kHid;
        float s = 0.0f;
        for (int u = 0; u < kHid; ++u) s += S.dz[r][u] * S.w2[u][v];
        S.z2[r][v] = s * gelu_grad(S.z1[r][v]);
    }
    __syncthreads();
    // dW1[u][c] = sum_r dZ1[r][u] x[r][c]; db1
    for (int i = tid; i < kHid * kIn; i += nth) {
        const int u = i / kIn, c = i % kIn;
        float s = 0.0f;
        for (int r = 0; r < kTrainRows; ++r) s += S.z2[r][u] * S.x[r][c];
        atomicAdd(&grads[kOffW1 + i], s);
    }
    if (tid < kHid) {
        float s = 0.0f;
        for (int r = 0; r < kTrainRows; ++r) s += S.z2[r][tid];
        atomicAdd(&grads[kOffB1 + tid], s);
    }
}

__global__ void k_adam(float *__restrict__ params, float *__restrict__ m, float *__restrict__ v,
                       const float *__restrict__ g, int step, float lr, uint16_t *__restrict__ w1b,
                       uint16_t *__restrict__ w2b, uint16_t *__restrict__ w3b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MG_MLP_PARAM_COUNT) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.0f - powf(b1, (float)step));
    const float vh = vi / (1.0f - powf(b2, (float)step));
    float p = params[i] - lr * mh / (sqrtf(vh) + eps);
    // inputs 54..63 are padding: keep their weights at zero
    if (i < kOffB1 && (i % kIn) >= MG_MLP_IN) p = 0.0f;
    params[i] = p;
    __nv_bfloat16 bv = __float2bfloat16_rn(p);
    const uint16_t bits = *reinterpret_cast<uint16_t *>(&bv);
    if (i < kOffB1)
        w1b[i - kOffW1] = bits;
    else if (i >= kOffW2 && i < kOffB2)
        w2b[i - kOffW2] = bits;
    else if (i >= kOffW3 && i < kOffB3)
        w3b[i - kOffW3] = bits;
}

}  // namespace mg

using namespace mg;

extern "C" int mg_mlp_forward(const uint16_t *features, int64_t n, const uint16_t *w1, const float *b1,
                              const uint16_t *w2, const float *b2, const uint16_t *w3, const float *b3,
                              const float *cell_side, float *out, float *seed_h, void *stream_) {
    if (!features || n <= 0 || !w1 || !b1 || !w2 || !b2 || !w3 || !b3 || !out) return MG_ERR_ARG;
    if (seed_h && !cell_side) return MG_ERR_ARG;
    int dev = 0, nsm = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t tiles = (n + 15) / 16;
    int64_t blocks = (tiles + 3) / 4;
    if (blocks > (int64_t)nsm * 16) blocks = (int64_t)nsm * 16;
    k_mlp_forward<<<(unsigned)blocks, 128, 0, as_stream(stream_)>>>(features, n, w1, b1, w2, b2, w3, b3,
                                                                     cell_side, out, seed_h);
    MG_CHECK_LAUNCH();
    return MG_OK;
}

extern "C" size_t mg_mlp_train_workspace_bytes(int64_t n) {
    return n > 0 ? align_up(sizeof(float) * MG_MLP_PARAM_COUNT) + 512 : 0;
}

extern "C" int mg_mlp_train_step(const uint16_t *features, const float *target, int64_t n, float *params,
                                 float *adam_m, float *adam_v, int32_t step, float lr, uint16_t *w1_bf16,
                                 uint16_t *w2_bf16, uint16_t *w3_bf16, float *loss_out, float *grads_out,
                                 void *workspace, size_t workspace_bytes, void *stream_) {
    if (!features || !target || n <= 0 || !params || !adam_m || !adam_v || step < 1 || !w1_bf16 || !w2_bf16 ||
        !w3_bf16 || !loss_out)
        return MG_ERR_ARG;
    if (workspace_bytes < mg_mlp_train_workspace_bytes(n)) return MG_ERR_ARG;
    cudaStream_t st = as_stream(stream_);
    Carve w(workspace, workspace_bytes);
    float *grads = w.take<float>(MG_MLP_PARAM_COUNT);
    if (!w.ok()) return MG_ERR_ARG;
    MG_CUDA(cudaMemsetAsync(grads, 0, sizeof(float) * MG_MLP_PARAM_COUNT, st));
    MG_CUDA(cudaMemsetAsync(loss_out, 0, sizeof(float), st));
    const size_t smem = sizeof(TrainSmem);
    MG_CUDA(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const unsigned blocks = (unsigned)((n + kTrainRows - 1) / kTrainRows);
    k_mlp_train<<<blocks, 256, smem, st>>>(features, target, n, params, grads, loss_out);
    MG_CHECK_LAUNCH();
    if (grads_out) MG_CUDA(cudaMemcpyAsync(grads_out, grads, sizeof(float) * MG_MLP_PARAM_COUNT,
                                           cudaMemcpyDeviceToDevice, st));
    k_adam<<<(MG_MLP_PARAM_COUNT + 255) / 256, 256, 0, st>>>(params, adam_m, adam_v, grads, step, lr, w1_bf16,
                                                              w2_bf16, w3_bf16);
    MG_CHECK_LAUNCH();
    return MG_OK;
}
