// mlp.cu -- the learned admissibility model: a 4-layer perceptron of hidden
// width 64 or 128, trained and evaluated by this library's own CUDA kernels.
//
// It maps the descriptors of a fragment-cluster pair (separation and radii in
// wavelengths, normal angles, visibility fraction) to the predicted log2 of
// the rank adaptive cross approximation needs for that block.  Blocks whose
// predicted rank is above the cut stay dense without an approximation
// attempt; the others are approximated with a rank cap derived from the
// prediction, and the exact tile still judges every approximation.
//
// Layers: 8 -> w -> w -> w -> 1 (w = 64 or 128), ReLU between.  Training in
// FP32 (weights, activations, gradients): mean-squared error on log2(rank),
// Adam; kernels: a shared-memory tiled dense layer (forward, input gradient,
// weight gradient), bias/ReLU epilogues, the loss gradient and the Adam
// update.  Inference: width 64 in FP32 on the CUDA cores (k_mlp_infer);
// width 128 with FP16 hidden layers on the tensor cores (k_mlp128_tc:
// tcgen05.mma, FP32 accumulators in tensor memory), the input and output
// layers in FP32.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "sonar_internal.h"
#include "tc05.cuh"

namespace sonar {
namespace {

constexpr int kIn = 8, kWidth = 64, kLayers = 4;  // kWidth: the CUDA-core inference kernel's width
constexpr int kWide = 128;                        // the tensor-core inference kernel's width
constexpr int kT = 16;  // tile of the dense-layer kernels

// Y[b, o] = sum_i X[b, i] W[o, i] + bias[o]  (optionally ReLU)
__global__ void k_dense_fwd(const float *X, const float *W, const float *bias, float *Y, int B, int in, int out,
                            int relu)
{
    __shared__ float sX[kT][kT + 1], sW[kT][kT + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int b = blockIdx.y * kT + ty, o = blockIdx.x * kT + tx;
    float acc = 0.0f;
    for (int k0 = 0; k0 < in; k0 += kT) {
        sX[ty][tx] = (b < B && k0 + tx < in) ? X[(size_t)b * in + k0 + tx] : 0.0f;
        const int ow = blockIdx.x * kT + ty;
        sW[ty][tx] = (ow < out && k0 + tx < in) ? W[(size_t)ow * in + k0 + tx] : 0.0f;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kT; ++k) acc = fmaf(sX[ty][k], sW[tx][k], acc);
        __syncthreads();
    }
    if (b < B && o < out) {
        float v = acc + bias[o];
        if (relu) v = fmaxf(v, 0.0f);
        Y[(size_t)b * out + o] = v;
    }
}

// dX[b, i] = sum_o dY[b, o] W[o, i]   (then masked by the ReLU of X's layer)
__global__ void k_dense_bwd_x(const float *dY, const float *W, const float *Xact, float *dX, int B, int in, int out,
                              int relu_mask)
{
    __shared__ float sD[kT][kT + 1], sW[kT][kT + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int b = blockIdx.y * kT + ty, i = blockIdx.x * kT + tx;
    float acc = 0.0f;
    for (int o0 = 0; o0 < out; o0 += kT) {
        sD[ty][tx] = (b < B && o0 + tx < out) ? dY[(size_t)b * out + o0 + tx] : 0.0f;
        const int iw = blockIdx.x * kT + tx;
        sW[ty][tx] = (o0 + ty < out && iw < in) ? W[(size_t)(o0 + ty) * in + iw] : 0.0f;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kT; ++k) acc = fmaf(sD[ty][k], sW[k][tx], acc);
        __syncthreads();
    }
    if (b < B && i < in) {
        if (relu_mask && !(Xact[(size_t)b * in + i] > 0.0f)) acc = 0.0f;
        dX[(size_t)b * in + i] = acc;
    }
}

// dW[o, i] = sum_b dY[b, o] X[b, i]
__global__ void k_dense_bwd_w(const float *dY, const float *X, float *dW, int B, int in, int out)
{
    __shared__ float sD[kT][kT + 1], sX[kT][kT + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int o = blockIdx.y * kT + ty, i = blockIdx.x * kT + tx;
    float acc = 0.0f;
    for (int b0 = 0; b0 < B; b0 += kT) {
        const int ob = blockIdx.y * kT + tx;
        sD[ty][tx] = (b0 + ty < B && ob < out) ? dY[(size_t)(b0 + ty) * out + ob] : 0.0f;
        sX[ty][tx] = (b0 + ty < B && i < in) ? X[(size_t)(b0 + ty) * in + i] : 0.0f;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kT; ++k) acc = fmaf(sD[k][ty], sX[k][tx], acc);
        __syncthreads();
    }
    if (o < out && i < in) dW[(size_t)o * in + i] = acc;
}

// db[o] = sum_b dY[b, o]
__global__ void k_bias_grad(const float *dY, float *db, int B, int out)
{
    const int o = blockIdx.x;
    float acc = 0.0f;
    for (int b = threadIdx.x; b < B; b += blockDim.x) acc += dY[(size_t)b * out + o];
    __shared__ float sv[8];
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) sv[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sv[w];
        db[o] = t;
    }
}

// mean-squared error: dY = 2 (y_hat - y) / B; per-sample squared error out
__global__ void k_mse(const float *yhat, const float *y, float *dY, float *se, int B)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const float d = yhat[b] - y[b];
    dY[b] = 2.0f * d / (float)B;
    se[b] = d * d;
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_gather(const float *X, const float *y, const int *idx, int B, float *Xb, float *yb)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const int i = idx[b];
#pragma unroll
    for (int k = 0; k < kIn; ++k) Xb[(size_t)b * kIn + k] = X[(size_t)i * kIn + k];
    yb[b] = y[i];
}

inline dim3 tiles(int cols, int rows) { return dim3((cols + kT - 1) / kT, (rows + kT - 1) / kT); }

// Inference of the whole network in one kernel: the parameters are staged
// once per CTA in shared memory (hidden layers transposed, [in][out], so
// that the 32 lanes of a warp read 32 consecutive outputs' weights), and each
// warp runs groups of kInferRows rows through the layers: lane l owns hidden
// units l, l + 32, ... (kUnits of them) of every row, the activations of the group
// pass between layers through the warp's shared-memory slice.
constexpr int kInferRows = 8;
constexpr int kUnits = kWidth / 32;  // hidden units per lane
constexpr int kInferWarps = 8;
constexpr size_t kInferSmem =
    sizeof(float) * ((size_t)kIn * kWidth + 2 * (size_t)kWidth * kWidth + 4 * kWidth + 1 +
                     (size_t)kInferWarps * kInferRows * (kWidth + kIn));

__global__ void __launch_bounds__(32 * kInferWarps) k_mlp_infer(const float *P, const float *X, int n, float *Y)
{
    extern __shared__ float sm[];
    float *W1 = sm;                                   // [kIn][kWidth]
    float *W2 = W1 + kIn * kWidth;                    // [kWidth][kWidth] (in, out)
    float *W3 = W2 + kWidth * kWidth;                 // [kWidth][kWidth]
    float *B1 = W3 + kWidth * kWidth, *B2 = B1 + kWidth, *B3 = B2 + kWidth, *W4 = B3 + kWidth, *B4 = W4 + kWidth;
    float *act = B4 + 1;                              // per warp: kInferRows x kWidth, then kInferRows x kIn
    // parameter vector: per layer W (out x in) then b (out)
    const float *p1 = P, *pb1 = p1 + kWidth * kIn, *p2 = pb1 + kWidth, *pb2 = p2 + kWidth * kWidth,
                *p3 = pb2 + kWidth, *pb3 = p3 + kWidth * kWidth, *p4 = pb3 + kWidth, *pb4 = p4 + kWidth;
    for (int e = threadIdx.x; e < kWidth * kWidth; e += blockDim.x) {
        const int o = e / kWidth, i = e - o * kWidth;
        W2[i * kWidth + o] = p2[e];
        W3[i * kWidth + o] = p3[e];
    }
    for (int e = threadIdx.x; e < kWidth * kIn; e += blockDim.x) {
        const int o = e / kIn, i = e - o * kIn;
        W1[i * kWidth + o] = p1[e];
    }
    for (int e = threadIdx.x; e < kWidth; e += blockDim.x) {
        B1[e] = pb1[e];
        B2[e] = pb2[e];
        B3[e] = pb3[e];
        W4[e] = p4[e];
    }
    if (threadIdx.x == 0) B4[0] = pb4[0];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *H = act + (size_t)warp * kInferRows * (kWidth + kIn);  // [kInferRows][kWidth]
    float *XI = H + kInferRows * kWidth;                          // [kInferRows][kIn]
    const int ngroups = (n + kInferRows - 1) / kInferRows;
    for (int g = blockIdx.x * kInferWarps + warp; g < ngroups; g += gridDim.x * kInferWarps) {
        const int r0 = g * kInferRows;
        for (int e = lane; e < kInferRows * kIn; e += 32) {
            const int r = r0 + e / kIn;
            XI[e] = r < n ? X[(size_t)r0 * kIn + e] : 0.0f;
        }
        __syncwarp();
        float acc[kInferRows][kUnits];
        // layer 1: 8 -> kWidth, ReLU
#pragma unroll
        for (int q = 0; q < kUnits; ++q) {
            const float b = B1[lane + 32 * q];
#pragma unroll
            for (int r = 0; r < kInferRows; ++r) acc[r][q] = b;
        }
#pragma unroll
        for (int i = 0; i < kIn; ++i) {
            float w[kUnits];
#pragma unroll
            for (int q = 0; q < kUnits; ++q) w[q] = W1[i * kWidth + lane + 32 * q];
#pragma unroll
            for (int r = 0; r < kInferRows; ++r) {
                const float x = XI[r * kIn + i];
#pragma unroll
                for (int q = 0; q < kUnits; ++q) acc[r][q] = fmaf(w[q], x, acc[r][q]);
            }
        }
        // layers 2 and 3: kWidth -> kWidth, ReLU
#pragma unroll 1
        for (int layer = 0; layer < 2; ++layer) {
            const float *W = layer == 0 ? W2 : W3, *Bv = layer == 0 ? B2 : B3;
            __syncwarp();
#pragma unroll
            for (int r = 0; r < kInferRows; ++r)
#pragma unroll
                for (int q = 0; q < kUnits; ++q) H[r * kWidth + lane + 32 * q] = fmaxf(acc[r][q], 0.0f);
            __syncwarp();
#pragma unroll
            for (int q = 0; q < kUnits; ++q) {
                const float b = Bv[lane + 32 * q];
#pragma unroll
                for (int r = 0; r < kInferRows; ++r) acc[r][q] = b;
            }
#pragma unroll 4
            for (int i = 0; i < kWidth; ++i) {
                float w[kUnits];
#pragma unroll
                for (int q = 0; q < kUnits; ++q) w[q] = W[i * kWidth + lane + 32 * q];
#pragma unroll
                for (int r = 0; r < kInferRows; ++r) {
                    const float h = H[r * kWidth + i];
#pragma unroll
                    for (int q = 0; q < kUnits; ++q) acc[r][q] = fmaf(w[q], h, acc[r][q]);
                }
            }
        }
        // output layer: kWidth -> 1
#pragma unroll
        for (int r = 0; r < kInferRows; ++r) {
            float v = 0.0f;
#pragma unroll
            for (int q = 0; q < kUnits; ++q) v = fmaf(W4[lane + 32 * q], fmaxf(acc[r][q], 0.0f), v);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0 && r0 + r < n) Y[r0 + r] = v + B4[0];
        }
        __syncwarp();
    }
}


// ---------------------------------------------------------------- width 128 on the tensor cores
// One CTA of 128 threads per tile of 128 rows (persistent over the tiles),
// thread r = row r = tensor-memory lane r.  Layer 1 (8 -> 128, FP32 on the
// CUDA cores) writes its ReLU output as FP16 into the A operand; each hidden
// layer is D (128 x 128, FP32 in tensor memory) = A (128 rows x 128, FP16)
// times W^T (W: 128 out x 128 in, FP16, staged once per CTA): eight
// tcgen05.mma of K = 16 issued by thread 0, completion on an mbarrier
// (bounded waits).  The accumulator comes back with tcgen05.ld, 16 columns at
// a time: bias and ReLU, then either the next layer's FP16 A operand or the
// output layer's dot product (FP32).  Operands in the no-swizzle K-major
// canonical layout: element (r, k) at (k / 8) * 2048 + r * 16 + (k % 8) * 2
// bytes.
constexpr int kTcRows = 128;
constexpr uint32_t kTcOpBytes = (uint32_t)kTcRows * kWide * 2;  // one FP16 operand, 32 KB
constexpr uint32_t kTcLbo = (uint32_t)kTcRows * 16;              // between the K core matrices
constexpr size_t kTcSmem = 3 * (size_t)kTcOpBytes + sizeof(float) * ((size_t)kIn * kWide + 4 * kWide + 4);
// instruction descriptor of kind::f16: FP32 accumulator, F16 A and B, both K-major, N = 128, M = 128
constexpr uint32_t kTcIdescF16 = (1u << 4) | ((uint32_t)(kWide >> 3) << 17) | ((uint32_t)(kTcRows >> 4) << 24);

__device__ __forceinline__ uint32_t tc_op_off(int r, int k8) { return (uint32_t)k8 * kTcLbo + (uint32_t)r * 16u; }

__device__ __forceinline__ uint4 pack_half8(const float *v)
{
    uint4 o;
    __half2 h;
    h = __floats2half2_rn(v[0], v[1]);
    o.x = *reinterpret_cast<uint32_t *>(&h);
    h = __floats2half2_rn(v[2], v[3]);
    o.y = *reinterpret_cast<uint32_t *>(&h);
    h = __floats2half2_rn(v[4], v[5]);
    o.z = *reinterpret_cast<uint32_t *>(&h);
    h = __floats2half2_rn(v[6], v[7]);
    o.w = *reinterpret_cast<uint32_t *>(&h);
    return o;
}

__global__ void __launch_bounds__(kTcRows, 1) k_mlp128_tc(const float *P, const float *X, int n, float *Y,
                                                          int *status)
{
    extern __shared__ __align__(1024) uint8_t smt[];
    uint8_t *sA = smt, *sB2 = smt + kTcOpBytes, *sB3 = smt + 2 * kTcOpBytes;
    float *W1 = reinterpret_cast<float *>(smt + 3 * kTcOpBytes);  // [kIn][kWide]
    float *B1 = W1 + kIn * kWide, *B2 = B1 + kWide, *B3 = B2 + kWide, *W4 = B3 + kWide, *B4 = W4 + kWide;
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) tmem_alloc(&tmem_base, kWide);
    if (tid == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // parameter vector: per layer W (out x in) then b (out)
    const float *p1 = P, *pb1 = p1 + kWide * kIn, *p2 = pb1 + kWide, *pb2 = p2 + kWide * kWide,
                *p3 = pb2 + kWide, *pb3 = p3 + kWide * kWide, *p4 = pb3 + kWide, *pb4 = p4 + kWide;
    for (int e = tid; e < kWide * kWide / 8; e += kTcRows) {
        const int o = e / (kWide / 8), k8 = e - o * (kWide / 8);
        float w[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) w[j] = p2[o * kWide + k8 * 8 + j];
        *reinterpret_cast<uint4 *>(sB2 + tc_op_off(o, k8)) = pack_half8(w);
#pragma unroll
        for (int j = 0; j < 8; ++j) w[j] = p3[o * kWide + k8 * 8 + j];
        *reinterpret_cast<uint4 *>(sB3 + tc_op_off(o, k8)) = pack_half8(w);
    }
    for (int e = tid; e < kWide * kIn; e += kTcRows) {
        const int o = e / kIn, i = e - o * kIn;
        W1[i * kWide + o] = p1[e];
    }
    for (int e = tid; e < kWide; e += kTcRows) {
        B1[e] = pb1[e];
        B2[e] = pb2[e];
        B3[e] = pb3[e];
        W4[e] = p4[e];
    }
    if (tid == 0) B4[0] = pb4[0];
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base, aA = smem_u32(sA), aB2 = smem_u32(sB2), aB3 = smem_u32(sB3);
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
    uint32_t commits = 0;
    bool ok = true;
    const int ntiles = (n + kTcRows - 1) / kTcRows;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int row = tile * kTcRows + tid;
        // layer 1: 8 -> 128, ReLU, FP16 into the A operand
        float x[kIn];
        if (row < n) {
            const float4 a = __ldg(reinterpret_cast<const float4 *>(X + (size_t)row * kIn));
            const float4 b = __ldg(reinterpret_cast<const float4 *>(X + (size_t)row * kIn) + 1);
            x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w; x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
        } else {
#pragma unroll
            for (int i = 0; i < kIn; ++i) x[i] = 0.0f;
        }
#pragma unroll 2
        for (int k8 = 0; k8 < kWide / 8; ++k8) {
            float h[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int o = k8 * 8 + j;
                float v = B1[o];
#pragma unroll
                for (int i = 0; i < kIn; ++i) v = fmaf(W1[i * kWide + o], x[i], v);
                h[j] = fmaxf(v, 0.0f);
            }
            *reinterpret_cast<uint4 *>(sA + tc_op_off(tid, k8)) = pack_half8(h);
        }
        float y = 0.0f;
        for (int layer = 0; layer < 2; ++layer) {
            // the A operand written by every thread -> visible to the tensor core
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
            if (tid == 0) {
                tc_fence_after();
                const uint32_t aB = layer ? aB3 : aB2;
#pragma unroll
                for (int ks = 0; ks < kWide / 16; ++ks)
                    mma_bf16(tmem, sdesc(aA + ks * 2 * kTcLbo, kTcLbo, 128), sdesc(aB + ks * 2 * kTcLbo, kTcLbo, 128),
                             kTcIdescF16, ks > 0 ? 1u : 0u);
                mma_commit(&bar);
            }
            ++commits;
            ok = __syncthreads_and(mbar_wait(&bar, (commits - 1) & 1u));
            if (!ok) break;
            tc_fence_after();
            const float *Bv = layer ? B3 : B2;
#pragma unroll 1
            for (int c = 0; c < kWide; c += 16) {
                float v[16];
                tmem_ld16(lane_addr + (uint32_t)c, v);
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j] + Bv[c + j], 0.0f);
                if (layer == 0) {
                    // the MMAs that read the A operand have completed: it becomes the next layer's input
                    *reinterpret_cast<uint4 *>(sA + tc_op_off(tid, c / 8)) = pack_half8(v);
                    *reinterpret_cast<uint4 *>(sA + tc_op_off(tid, c / 8 + 1)) = pack_half8(v + 8);
                } else {
#pragma unroll
                    for (int j = 0; j < 16; ++j) y = fmaf(W4[c + j], v[j], y);
                }
            }
            tc_fence_before();
        }
        if (ok && row < n) Y[row] = y + B4[0];
    }
    // a timed-out wait may leave MMAs in flight: wait for the last commit
    // (bounded again) before the tensor memory is released; if that runs out
    // too, the tensor memory stays allocated and the status says so (2)
    bool drained = true;
    if (!ok && commits > 0) drained = __syncthreads_and(mbar_wait(&bar, (commits - 1) & 1u));
    if (!ok && tid == 0) atomicExch(status, drained ? 1 : 2);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0 && drained) tmem_dealloc(tmem, kWide);
}

}  // namespace

// ---------------------------------------------------------------- host model
struct Mlp {
    int width = kWidth;
    int dims[kLayers + 1] = {kIn, kWidth, kWidth, kWidth, 1};
    // flat parameter vector: for each layer W (out x in) then b (out)
    std::vector<size_t> woff, boff;
    size_t nparam = 0;
    float *d_p = nullptr, *d_g = nullptr, *d_m = nullptr, *d_v = nullptr;
    int *d_status = nullptr;  // tensor-core inference: 1 (2) when a wait ran out (and the tensor memory was kept)
    int adam_t = 0;
    bool ready = false;

    void layout()
    {
        dims[1] = dims[2] = dims[3] = width;
        woff.assign(kLayers, 0);
        boff.assign(kLayers, 0);
        size_t o = 0;
        for (int l = 0; l < kLayers; ++l) {
            woff[l] = o;
            o += (size_t)dims[l + 1] * dims[l];
            boff[l] = o;
            o += dims[l + 1];
        }
        nparam = o;
    }
    void release()
    {
        for (float **q : {&d_p, &d_g, &d_m, &d_v})
            if (*q) {
                cudaFree(*q);
                *q = nullptr;
            }
        if (d_status) cudaFree(d_status);
        d_status = nullptr;
        ready = false;
    }
};

static Mlp g_mlp;

// Hidden width 64 or 128; the parameters are dropped (initialise or load new ones).
cudaError_t mlp_set_width(int width)
{
    if (width != kWidth && width != kWide) return cudaErrorInvalidValue;
    if (width == g_mlp.width) return cudaSuccess;
    g_mlp.release();
    g_mlp.width = width;
    g_mlp.layout();
    return cudaSuccess;
}

int mlp_width() { return g_mlp.width; }

// Status of the tensor-core inference since the last call (0: fine), reset.
int mlp_take_status()
{
    if (!g_mlp.d_status) return 0;
    int v = 0;
    if (cudaMemcpy(&v, g_mlp.d_status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    if (v) cudaMemset(g_mlp.d_status, 0, sizeof(int));
    return v;
}

static cudaError_t mlp_alloc()
{
    if (g_mlp.d_p) return cudaSuccess;
    g_mlp.layout();
    cudaError_t e = cudaMalloc(&g_mlp.d_p, g_mlp.nparam * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&g_mlp.d_g, g_mlp.nparam * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&g_mlp.d_m, g_mlp.nparam * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&g_mlp.d_v, g_mlp.nparam * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&g_mlp.d_status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(g_mlp.d_status, 0, sizeof(int));
    return e;
}

size_t mlp_param_count()
{
    g_mlp.layout();
    return g_mlp.nparam;
}

// He-uniform initialisation from a seed (host), zero Adam state.
cudaError_t mlp_init(unsigned seed)
{
    cudaError_t e = mlp_alloc();
    if (e != cudaSuccess) return e;
    std::vector<float> p(g_mlp.nparam, 0.0f);
    std::mt19937 rng(seed);
    for (int l = 0; l < kLayers; ++l) {
        const float lim = std::sqrt(6.0f / (float)g_mlp.dims[l]);
        std::uniform_real_distribution<float> u(-lim, lim);
        for (size_t k = 0; k < (size_t)g_mlp.dims[l + 1] * g_mlp.dims[l]; ++k) p[g_mlp.woff[l] + k] = u(rng);
    }
    e = cudaMemcpy(g_mlp.d_p, p.data(), p.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(g_mlp.d_m, 0, g_mlp.nparam * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(g_mlp.d_v, 0, g_mlp.nparam * sizeof(float));
    g_mlp.adam_t = 0;
    g_mlp.ready = e == cudaSuccess;
    return e;
}

cudaError_t mlp_set_params(const float *p, size_t n)
{
    cudaError_t e = mlp_alloc();
    if (e != cudaSuccess) return e;
    if (n != g_mlp.nparam) return cudaErrorInvalidValue;
    e = cudaMemcpy(g_mlp.d_p, p, n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(g_mlp.d_m, 0, n * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(g_mlp.d_v, 0, n * sizeof(float));
    g_mlp.adam_t = 0;
    g_mlp.ready = e == cudaSuccess;
    return e;
}

cudaError_t mlp_get_params(float *p, size_t n)
{
    if (!g_mlp.ready || n != g_mlp.nparam) return cudaErrorInvalidValue;
    return cudaMemcpy(p, g_mlp.d_p, n * sizeof(float), cudaMemcpyDeviceToHost);
}

bool mlp_ready() { return g_mlp.ready; }

// Activations of a batch: A[0] = X (B x 8), A[l] (B x dims[l]), A[4] = y_hat.
struct Acts {
    float *a[kLayers + 1] = {nullptr};
    float *d[kLayers + 1] = {nullptr};
    int B = 0;
    cudaError_t alloc(int b)
    {
        release();
        B = b;
        for (int l = 0; l <= kLayers; ++l) {
            cudaError_t e = cudaMalloc(&a[l], (size_t)b * g_mlp.dims[l] * sizeof(float));
            if (e == cudaSuccess) e = cudaMalloc(&d[l], (size_t)b * g_mlp.dims[l] * sizeof(float));
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    void release()
    {
        for (int l = 0; l <= kLayers; ++l) {
            if (a[l]) cudaFree(a[l]);
            if (d[l]) cudaFree(d[l]);
            a[l] = d[l] = nullptr;
        }
    }
};

static void forward(Acts &A, int B, cudaStream_t s)
{
    for (int l = 0; l < kLayers; ++l) {
        const int in = g_mlp.dims[l], out = g_mlp.dims[l + 1];
        k_dense_fwd<<<tiles(out, B), dim3(kT, kT), 0, s>>>(A.a[l], g_mlp.d_p + g_mlp.woff[l], g_mlp.d_p + g_mlp.boff[l],
                                                            A.a[l + 1], B, in, out, l + 1 < kLayers);
    }
}

// gradient of the mean squared error of one batch into d_g; per-sample
// squared errors into se (device, B floats)
static void backward(Acts &A, const float *y, float *se, int B, cudaStream_t s)
{
    k_mse<<<(B + 255) / 256, 256, 0, s>>>(A.a[kLayers], y, A.d[kLayers], se, B);
    for (int l = kLayers - 1; l >= 0; --l) {
        const int in = g_mlp.dims[l], out = g_mlp.dims[l + 1];
        k_dense_bwd_w<<<tiles(in, out), dim3(kT, kT), 0, s>>>(A.d[l + 1], A.a[l], g_mlp.d_g + g_mlp.woff[l], B, in,
                                                              out);
        k_bias_grad<<<out, 256, 0, s>>>(A.d[l + 1], g_mlp.d_g + g_mlp.boff[l], B, out);
        if (l > 0)
            k_dense_bwd_x<<<tiles(in, B), dim3(kT, kT), 0, s>>>(A.d[l + 1], g_mlp.d_p + g_mlp.woff[l], A.a[l],
                                                                A.d[l], B, in, out, 1);
    }
}

// One forward/backward pass; gradient and loss to the host (gradient checks).
cudaError_t mlp_grad(const float *X, const float *y, int B, float *grad, float *loss)
{
    if (!g_mlp.ready || B <= 0) return cudaErrorInvalidValue;
    Acts A;
    float *d_y = nullptr, *d_se = nullptr;
    cudaError_t e = A.alloc(B);
    if (e == cudaSuccess) e = cudaMalloc(&d_y, B * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&d_se, B * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(A.a[0], X, (size_t)B * kIn * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_y, y, B * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        forward(A, B, 0);
        backward(A, d_y, d_se, B, 0);
        e = cudaGetLastError();
    }
    std::vector<float> se(B);
    if (e == cudaSuccess) e = cudaMemcpy(grad, g_mlp.d_g, g_mlp.nparam * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(se.data(), d_se, B * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) {
        double t = 0.0;
        for (float v : se) t += v;
        *loss = (float)(t / B);
    }
    A.release();
    if (d_y) cudaFree(d_y);
    if (d_se) cudaFree(d_se);
    return e;
}

// Adam training on device arrays (n rows of 8 descriptors, n labels):
// mini-batches in a seeded shuffled order, gathered on the device.  Returns
// the mean squared error of the last epoch.
cudaError_t mlp_train_dev(const float *d_X, const float *d_y, int n, int epochs, int batch, float lr, unsigned seed,
                          float *last_loss, cudaStream_t s)
{
    if (!g_mlp.ready || n <= 0 || epochs < 0) return cudaErrorInvalidValue;
    batch = std::max(1, std::min(batch, n));
    const int nb = n / batch;
    float *d_by = nullptr, *d_se = nullptr;
    int *d_idx = nullptr;
    Acts A;
    cudaError_t e = cudaMalloc(&d_se, (size_t)nb * batch * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&d_by, (size_t)batch * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&d_idx, (size_t)n * sizeof(int));
    if (e == cudaSuccess) e = A.alloc(batch);
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::mt19937 rng(seed);
    std::vector<float> se((size_t)nb * batch);
    double epoch_loss = 0.0;
    for (int ep = 0; ep < epochs && e == cudaSuccess; ++ep) {
        std::shuffle(order.begin(), order.end(), rng);
        e = cudaMemcpyAsync(d_idx, order.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s);
        for (int k = 0; k < nb && e == cudaSuccess; ++k) {
            k_gather<<<(batch + 255) / 256, 256, 0, s>>>(d_X, d_y, d_idx + (size_t)k * batch, batch, A.a[0], d_by);
            forward(A, batch, s);
            backward(A, d_by, d_se + (size_t)k * batch, batch, s);
            ++g_mlp.adam_t;
            const float b1 = 0.9f, b2 = 0.999f;
            const float c1 = 1.0f - std::pow(b1, (float)g_mlp.adam_t), c2 = 1.0f - std::pow(b2, (float)g_mlp.adam_t);
            k_adam<<<(unsigned)((g_mlp.nparam + 255) / 256), 256, 0, s>>>(
                g_mlp.d_p, g_mlp.d_g, g_mlp.d_m, g_mlp.d_v, (int)g_mlp.nparam, lr, b1, b2, 1e-8f, c1, c2);
        }
        // the order vector must stay unchanged until its upload has completed
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    if (e == cudaSuccess && epochs > 0 && nb > 0) {
        e = cudaMemcpy(se.data(), d_se, se.size() * sizeof(float), cudaMemcpyDeviceToHost);
        for (float v : se) epoch_loss += v;
        epoch_loss /= (double)se.size();
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (last_loss) *last_loss = (float)epoch_loss;
    A.release();
    if (d_se) cudaFree(d_se);
    if (d_by) cudaFree(d_by);
    if (d_idx) cudaFree(d_idx);
    return e;
}

// The same from host arrays.
cudaError_t mlp_train(const float *X, const float *y, int n, int epochs, int batch, float lr, unsigned seed,
                      float *last_loss)
{
    if (!g_mlp.ready || n <= 0) return cudaErrorInvalidValue;
    float *d_X = nullptr, *d_y = nullptr;
    cudaError_t e = cudaMalloc(&d_X, (size_t)n * kIn * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&d_y, (size_t)n * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(d_X, X, (size_t)n * kIn * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_y, y, (size_t)n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = mlp_train_dev(d_X, d_y, n, epochs, batch, lr, seed, last_loss, 0);
    if (d_X) cudaFree(d_X);
    if (d_y) cudaFree(d_y);
    return e;
}

// Predicted log2(1 + rank) of n descriptor rows (device arrays, X 16-byte
// aligned), on stream s, by the fused inference kernel of the width.
cudaError_t mlp_infer_dev(const float *dX, int n, float *dY, cudaStream_t s)
{
    if (!g_mlp.ready) return cudaErrorInvalidValue;
    if (n <= 0) return cudaSuccess;
    if (g_mlp.width == kWide) {
        static bool attr_tc = false;
        if (!attr_tc) {
            const cudaError_t e =
                cudaFuncSetAttribute(k_mlp128_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
            if (e != cudaSuccess) return e;
            attr_tc = true;
        }
        int dev = 0, nsm = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        const int ntiles = (n + kTcRows - 1) / kTcRows;
        k_mlp128_tc<<<std::max(1, std::min(nsm, ntiles)), kTcRows, kTcSmem, s>>>(g_mlp.d_p, dX, n, dY, g_mlp.d_status);
        return cudaGetLastError();
    }
    static bool attr = false;
    if (!attr) {
        const cudaError_t e =
            cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int groups = (n + kInferRows - 1) / kInferRows;
    const int grid = std::max(1, std::min(nsm, (groups + kInferWarps - 1) / kInferWarps));
    k_mlp_infer<<<grid, 32 * kInferWarps, kInferSmem, s>>>(g_mlp.d_p, dX, n, dY);
    return cudaGetLastError();
}

}  // namespace sonar
