// Learned path guiding on the tensor cores: fused encoding + MLP forward/backward with weight
// and hash-grid gradients, Adam, and mixture inference. The model is defined in lf_guide.cuh.
//
// Tensor-core mapping: one warp owns a tile of 16 samples and runs every layer as
// mma.sync.m16n8k16 (FP16 operands, FP32 accumulators). A layer's output fragments become the
// next layer's input fragments in registers (two adjacent 16x8 accumulator tiles form one
// 16x16 operand tile), so activations never leave the warp during the forward pass; the
// backward pass reuses them for the ReLU masks. Weight gradients (out x in, summed over the 16
// samples) are a second mma with the samples as the reduction dimension, staged through the
// warp's shared memory and summed per block in shared FP32 before one global add per weight.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "lf_guide.cuh"
#include "lf_internal.h"

namespace lfd
{
namespace guide
{
namespace
{
constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarps = 4;            // warps per block
constexpr int kLd = 72;              // halves per staging row (64 + 8 pad)
// Inference keeps the weights in shared memory with rows padded to kLd halves as well: with
// 64-half rows the B-fragment loads of the 8 row groups of a warp all hit the same banks.
constexpr int kWRows = 3 * 64 + kOut;
constexpr int kWPadded = kWRows * kLd;
constexpr int kInferWarps = 8;        // warps per inference block (a lighter stage than training's)

struct WarpStage
{
    __half x[16 * kLd];              // inputs
    __half a[16 * kLd];              // activations
    __half g[16 * kLd];              // gradients
    float out[16 * kOut];            // MLP outputs
    float dx[16 * 32];               // gradient of the grid features
};

struct InferStage
{
    __half x[16 * kLd];              // inputs
    float out[16 * kOut];            // MLP outputs
};

struct SharedTrain
{
    __half W[kWeights];              // [out][in]
    __half WT[kWeights];             // W1^T, W2^T, W3^T [in][out] 64x64; W4^T [in][out] 64x48
    float dW[kWeights];              // block sums of weight gradients
    WarpStage ws[kWarps];
};

__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack(float lo, float hi)
{
    __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
}

__device__ __forceinline__ uint32_t pack_h(__half lo, __half hi)
{
    return (uint32_t)__half_as_ushort(lo) | ((uint32_t)__half_as_ushort(hi) << 16);
}

__device__ __forceinline__ float lo_f(uint32_t v) { return __half2float(__ushort_as_half((unsigned short)(v & 0xffffu))); }
__device__ __forceinline__ float hi_f(uint32_t v) { return __half2float(__ushort_as_half((unsigned short)(v >> 16))); }

__device__ __forceinline__ uint32_t ld32(const __half* p) { return *reinterpret_cast<const uint32_t*>(p); }

// C[j] (16 x 8NT, FP32) = A (16 x 16KT) * B, B[k][n] = M[n * ldm + k] (M row-major [n][k]).
template <int KT, int NT>
__device__ __forceinline__ void gemm_rows(const uint32_t A[KT][4], const __half* M, int ldm, float C[NT][4])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int j = 0; j < NT; ++j)
    {
        C[j][0] = C[j][1] = C[j][2] = C[j][3] = 0.f;
        const __half* row = M + (j * 8 + g) * ldm;
#pragma unroll
        for (int kt = 0; kt < KT; ++kt) mma16816(C[j], A[kt], ld32(row + kt * 16 + t * 2), ld32(row + kt * 16 + 8 + t * 2));
    }
}

// Accumulator tiles (16 x 64) -> operand tiles, through ReLU.
__device__ __forceinline__ void relu_operand(const float C[8][4], uint32_t A[4][4])
{
#pragma unroll
    for (int kt = 0; kt < 4; ++kt)
    {
        A[kt][0] = pack(fmaxf(C[2 * kt][0], 0.f), fmaxf(C[2 * kt][1], 0.f));
        A[kt][1] = pack(fmaxf(C[2 * kt][2], 0.f), fmaxf(C[2 * kt][3], 0.f));
        A[kt][2] = pack(fmaxf(C[2 * kt + 1][0], 0.f), fmaxf(C[2 * kt + 1][1], 0.f));
        A[kt][3] = pack(fmaxf(C[2 * kt + 1][2], 0.f), fmaxf(C[2 * kt + 1][3], 0.f));
    }
}

// Gradient accumulator tiles -> operand tiles, masked by the layer's ReLU (H > 0).
__device__ __forceinline__ void masked_operand(const float C[8][4], const uint32_t H[4][4], uint32_t G[4][4])
{
#pragma unroll
    for (int kt = 0; kt < 4; ++kt)
    {
        const float* c0 = C[2 * kt];
        const float* c1 = C[2 * kt + 1];
        G[kt][0] = pack(lo_f(H[kt][0]) > 0.f ? c0[0] : 0.f, hi_f(H[kt][0]) > 0.f ? c0[1] : 0.f);
        G[kt][1] = pack(lo_f(H[kt][1]) > 0.f ? c0[2] : 0.f, hi_f(H[kt][1]) > 0.f ? c0[3] : 0.f);
        G[kt][2] = pack(lo_f(H[kt][2]) > 0.f ? c1[0] : 0.f, hi_f(H[kt][2]) > 0.f ? c1[1] : 0.f);
        G[kt][3] = pack(lo_f(H[kt][3]) > 0.f ? c1[2] : 0.f, hi_f(H[kt][3]) > 0.f ? c1[3] : 0.f);
    }
}

// Operand tiles (16 x 16KT) -> row-major staging [16][kLd].
template <int KT>
__device__ __forceinline__ void stage(const uint32_t A[KT][4], __half* s)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int kt = 0; kt < KT; ++kt)
    {
        *reinterpret_cast<uint32_t*>(s + g * kLd + kt * 16 + t * 2) = A[kt][0];
        *reinterpret_cast<uint32_t*>(s + (g + 8) * kLd + kt * 16 + t * 2) = A[kt][1];
        *reinterpret_cast<uint32_t*>(s + g * kLd + kt * 16 + 8 + t * 2) = A[kt][2];
        *reinterpret_cast<uint32_t*>(s + (g + 8) * kLd + kt * 16 + 8 + t * 2) = A[kt][3];
    }
}

template <int KT>
__device__ __forceinline__ void load_operand(const __half* s, uint32_t A[KT][4])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int kt = 0; kt < KT; ++kt)
    {
        A[kt][0] = ld32(s + g * kLd + kt * 16 + t * 2);
        A[kt][1] = ld32(s + (g + 8) * kLd + kt * 16 + t * 2);
        A[kt][2] = ld32(s + g * kLd + kt * 16 + 8 + t * 2);
        A[kt][3] = ld32(s + (g + 8) * kLd + kt * 16 + 8 + t * 2);
    }
}

// dW[m][n] += sum over the 16 samples of G[s][m] * H[s][n]; G, H staged row-major [16][kLd].
template <int MT>
__device__ __forceinline__ void weight_grad(const __half* sG, const __half* sH, float* dW, int ldw)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
    {
        const int m = mt * 16 + g;
        uint32_t a[4];
        a[0] = pack_h(sG[(t * 2) * kLd + m], sG[(t * 2 + 1) * kLd + m]);
        a[1] = pack_h(sG[(t * 2) * kLd + m + 8], sG[(t * 2 + 1) * kLd + m + 8]);
        a[2] = pack_h(sG[(t * 2 + 8) * kLd + m], sG[(t * 2 + 9) * kLd + m]);
        a[3] = pack_h(sG[(t * 2 + 8) * kLd + m + 8], sG[(t * 2 + 9) * kLd + m + 8]);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
        {
            const int n = nt * 8 + g;
            const uint32_t b0 = pack_h(sH[(t * 2) * kLd + n], sH[(t * 2 + 1) * kLd + n]);
            const uint32_t b1 = pack_h(sH[(t * 2 + 8) * kLd + n], sH[(t * 2 + 9) * kLd + n]);
            float d[4] = {0.f, 0.f, 0.f, 0.f};
            mma16816(d, a, b0, b1);
            const int col = nt * 8 + t * 2;
            atomicAdd(&dW[m * ldw + col], d[0]);
            atomicAdd(&dW[m * ldw + col + 1], d[1]);
            atomicAdd(&dW[(m + 8) * ldw + col], d[2]);
            atomicAdd(&dW[(m + 8) * ldw + col + 1], d[3]);
        }
    }
}

// Encodes the 16 samples of a tile into x (row-major halves). Lane: sample lane & 15, half
// lane >> 4: levels 0..3 + outgoing-direction blobs, or levels 4..7 + normal blobs.
__device__ __forceinline__ void encode_tile(const Net& net, const float* p, const float* wo, const float* n, bool valid,
                                            __half* x)
{
    const int lane = threadIdx.x & 31, s = lane & 15, h = lane >> 4;
    __half* row = x + s * kLd;
    if (!valid)
    {
        for (int f = 0; f < 16; ++f) row[h * 16 + f] = __float2half(0.f);
        for (int f = 0; f < 16; ++f) row[32 + h * 16 + f] = __float2half(0.f);
        return;
    }
    float p01[3];
    position01(net, p, p01);
    for (int l = h * 4; l < h * 4 + 4; ++l)
    {
        float acc[4];
        level_features(net, l, p01, acc);
        for (int f = 0; f < 4; ++f) row[l * 4 + f] = __float2half(acc[f]);
    }
    const float* d = h == 0 ? wo : n;
    float th, ph;
    sph01(d[0], d[1], d[2], &th, &ph);
    for (int k = 0; k < kBlobBins; ++k)
    {
        row[32 + h * 16 + k] = __float2half(blob(th, k));
        row[32 + h * 16 + 8 + k] = __float2half(blob(ph, k));
    }
}

}

// One pass over n training samples: adds the per-sample gradients (not divided by n) of every
// weight into gW and of every grid parameter into gGrid, and the summed loss into loss.
__global__ void __launch_bounds__(kWarps * 32) guide_train_kernel(Net net, const float* samples, int n, float* gW,
                                                                  float* gGrid, float* loss)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SharedTrain& S = *reinterpret_cast<SharedTrain*>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    for (int i = threadIdx.x; i < kWeights; i += blockDim.x)
    {
        S.W[i] = net.W[i];
        S.dW[i] = 0.f;
    }
    __syncthreads();
    // transposes: layers 1..3 [in][out] 64x64, layer 4 [in][out] 64x48
    for (int i = threadIdx.x; i < kWeights; i += blockDim.x)
    {
        if (i < kW4)
        {
            const int l = i / 4096, r = i % 4096, o = r / 64, in = r % 64;
            S.WT[l * 4096 + in * 64 + o] = S.W[i];
        }
        else
        {
            const int r = i - kW4, o = r / 64, in = r % 64;
            S.WT[kW4 + in * kOut + o] = S.W[i];
        }
    }
    __syncthreads();
    WarpStage& ws = S.ws[warp];
    float lossSum = 0.f;
    const int tiles = (n + 15) / 16;
    for (int tile = blockIdx.x * kWarps + warp; tile < tiles; tile += gridDim.x * kWarps)
    {
        const int s = tile * 16 + (lane & 15);
        const bool valid = s < n;
        const float* rec = samples + (size_t)(valid ? s : 0) * kSampleFloats;
        encode_tile(net, rec, rec + 3, rec + 6, valid, ws.x);
        __syncwarp();
        uint32_t X[4][4], H1[4][4], H2[4][4], H3[4][4];
        float C[8][4];
        load_operand<4>(ws.x, X);
        gemm_rows<4, 8>(X, S.W + kW1, 64, C);
        relu_operand(C, H1);
        gemm_rows<4, 8>(H1, S.W + kW2, 64, C);
        relu_operand(C, H2);
        gemm_rows<4, 8>(H2, S.W + kW3, 64, C);
        relu_operand(C, H3);
        float Co[6][4];
        gemm_rows<4, 6>(H3, S.W + kW4, 64, Co);
#pragma unroll
        for (int j = 0; j < 6; ++j)
        {
            ws.out[g * kOut + j * 8 + t * 2] = Co[j][0];
            ws.out[g * kOut + j * 8 + t * 2 + 1] = Co[j][1];
            ws.out[(g + 8) * kOut + j * 8 + t * 2] = Co[j][2];
            ws.out[(g + 8) * kOut + j * 8 + t * 2 + 1] = Co[j][3];
        }
        __syncwarp();
        if (lane < 16)
        {
            float d_out[40];
            float l = 0.f;
            if (valid)
                l = sample_loss_grad(ws.out + lane * kOut, rec + 9, rec[12], d_out);
            else
                for (int k = 0; k < 40; ++k) d_out[k] = 0.f;
            lossSum += l;
            for (int k = 0; k < 40; ++k) ws.g[lane * kLd + k] = __float2half(d_out[k]);
            for (int k = 40; k < kOut; ++k) ws.g[lane * kLd + k] = __float2half(0.f);
        }
        __syncwarp();
        // layer 4: dW4 += G4^T H3, dH3 = G4 W4
        uint32_t G4[3][4];
        load_operand<3>(ws.g, G4);
        stage<4>(H3, ws.a);
        __syncwarp();
        weight_grad<3>(ws.g, ws.a, S.dW + kW4, 64);
        gemm_rows<3, 8>(G4, S.WT + kW4, kOut, C);
        uint32_t G[4][4];
        masked_operand(C, H3, G);
        __syncwarp();
        // layer 3
        stage<4>(G, ws.g);
        stage<4>(H2, ws.a);
        __syncwarp();
        weight_grad<4>(ws.g, ws.a, S.dW + kW3, 64);
        gemm_rows<4, 8>(G, S.WT + kW3, 64, C);
        masked_operand(C, H2, G);
        __syncwarp();
        // layer 2
        stage<4>(G, ws.g);
        stage<4>(H1, ws.a);
        __syncwarp();
        weight_grad<4>(ws.g, ws.a, S.dW + kW2, 64);
        gemm_rows<4, 8>(G, S.WT + kW2, 64, C);
        masked_operand(C, H1, G);
        __syncwarp();
        // layer 1 and the input gradient (grid features only: inputs 0..31)
        stage<4>(G, ws.g);
        __syncwarp();
        weight_grad<4>(ws.g, ws.x, S.dW + kW1, 64);
        float Cx[4][4];
        gemm_rows<4, 4>(G, S.WT + kW1, 64, Cx);
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
            ws.dx[g * 32 + j * 8 + t * 2] = Cx[j][0];
            ws.dx[g * 32 + j * 8 + t * 2 + 1] = Cx[j][1];
            ws.dx[(g + 8) * 32 + j * 8 + t * 2] = Cx[j][2];
            ws.dx[(g + 8) * 32 + j * 8 + t * 2 + 1] = Cx[j][3];
        }
        __syncwarp();
        if (valid)
        {
            float p01[3];
            position01(net, rec, p01);
            const int sl = lane & 15, h = lane >> 4;
            for (int l = h * 4; l < h * 4 + 4; ++l)
            {
                uint32_t idx[8];
                float w[8];
                grid_corners(net.res[l], p01, idx, w);
                float* gt = gGrid + (size_t)l * kT * kFeatures;
                for (int c = 0; c < 8; ++c)
                    for (int f = 0; f < 4; ++f) atomicAdd(&gt[(size_t)idx[c] * kFeatures + f], w[c] * ws.dx[sl * 32 + l * 4 + f]);
            }
        }
        __syncwarp();
    }
    for (int off = 16; off > 0; off >>= 1) lossSum += __shfl_xor_sync(kFull, lossSum, off);
    if (lane == 0 && lossSum != 0.f) atomicAdd(loss, lossSum);
    __syncthreads();
    for (int i = threadIdx.x; i < kWeights; i += blockDim.x)
        if (S.dW[i] != 0.f) atomicAdd(&gW[i], S.dW[i]);
}

// Adam over FP32 master parameters (gradients scaled by gradScale, then cleared), refreshing
// the FP16 working copy.
__global__ void guide_adam_kernel(float* master, __half* work, float* m, float* v, float* grad, int n, float lr,
                                  float b1, float b2, float eps, float c1, float c2, float gradScale)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const float gr = grad[i] * gradScale;
        grad[i] = 0.f;
        const float mi = b1 * m[i] + (1.f - b1) * gr;
        const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
        m[i] = mi;
        v[i] = vi;
        const float p = master[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        master[i] = p;
        work[i] = __float2half(p);
    }
}

// Mixture of every query (sample records: p, wo, n) in the compact form used for sampling:
// per lobe mu xyz, kappa and the cumulative lobe weight.
__global__ void __launch_bounds__(kInferWarps * 32) guide_infer_kernel(Net net, const float* queries, int n,
                                                                       const int* nDev, float* mix)
{
    if (nDev) n = *nDev;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __half* W = reinterpret_cast<__half*>(smem_raw);
    InferStage* stages = reinterpret_cast<InferStage*>(smem_raw + sizeof(__half) * kWPadded);
    for (int i = threadIdx.x; i < kWeights; i += blockDim.x) W[(i / 64) * kLd + (i % 64)] = net.W[i];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    InferStage& ws = stages[warp];
    const int tiles = (n + 15) / 16;
    for (int tile = blockIdx.x * kInferWarps + warp; tile < tiles; tile += gridDim.x * kInferWarps)
    {
        const int s = tile * 16 + (lane & 15);
        const bool valid = s < n;
        const float* rec = queries + (size_t)(valid ? s : 0) * kSampleFloats;
        encode_tile(net, rec, rec + 3, rec + 6, valid, ws.x);
        __syncwarp();
        uint32_t A[4][4], H[4][4];
        float C[8][4];
        load_operand<4>(ws.x, A);
        gemm_rows<4, 8>(A, W + 0 * 64 * kLd, kLd, C);
        relu_operand(C, H);
        gemm_rows<4, 8>(H, W + 1 * 64 * kLd, kLd, C);
        relu_operand(C, A);
        gemm_rows<4, 8>(A, W + 2 * 64 * kLd, kLd, C);
        relu_operand(C, H);
        float Co[6][4];
        gemm_rows<4, 6>(H, W + 3 * 64 * kLd, kLd, Co);
#pragma unroll
        for (int j = 0; j < 6; ++j)
        {
            ws.out[g * kOut + j * 8 + t * 2] = Co[j][0];
            ws.out[g * kOut + j * 8 + t * 2 + 1] = Co[j][1];
            ws.out[(g + 8) * kOut + j * 8 + t * 2] = Co[j][2];
            ws.out[(g + 8) * kOut + j * 8 + t * 2 + 1] = Co[j][3];
        }
        __syncwarp();
        if (lane < 16 && valid)
        {
            const float* out = ws.out + lane * kOut;
            float* dst = mix + (size_t)s * kMixFloats;
            float mx = -1e30f;
            for (int i = 0; i < kLobes; ++i) mx = fmaxf(mx, out[5 * i + 4]);
            float es = 0.f, e[kLobes];
            for (int i = 0; i < kLobes; ++i)
            {
                e[i] = __expf(out[5 * i + 4] - mx);
                es += e[i];
            }
            const float invEs = 1.f / es;
            float cum = 0.f;
            for (int i = 0; i < kLobes; ++i)
            {
                float mu[3], k;
                lobe_params(out + 5 * i, mu, &k);
                cum += e[i] * invEs;
                dst[5 * i + 0] = mu[0];
                dst[5 * i + 1] = mu[1];
                dst[5 * i + 2] = mu[2];
                dst[5 * i + 3] = k;
                dst[5 * i + 4] = i == kLobes - 1 ? 1.f : cum;
            }
        }
        __syncwarp();
    }
}

__global__ void guide_pdf_kernel(const float* mix, const float* queries, int n, float* pdf)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const float* d = queries + (size_t)i * kSampleFloats + 9;
        pdf[i] = mix_pdf(mix + (size_t)i * kMixFloats, d[0], d[1], d[2]);
    }
}

__global__ void to_half_kernel(const float* a, __half* b, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = __float2half(a[i]);
}

size_t train_smem() { return sizeof(SharedTrain); }
size_t infer_smem() { return sizeof(__half) * kWPadded + sizeof(InferStage) * kInferWarps; }

int launch_infer(const Net& net, const float* queries, const int* nDev, int cap, float* mix, cudaStream_t st)
{
    static bool attr = false;
    if (!attr)
    {
        cudaFuncSetAttribute(guide_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)infer_smem());
        attr = true;
    }
    int sms = 1, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int tiles = (cap + 15) / 16;
    const int perSm = occupancy_blocks_per_sm((const void*)guide_infer_kernel, kInferWarps * 32, infer_smem());
    const int blocks = std::max(1, std::min(sms * perSm, (tiles + kInferWarps - 1) / kInferWarps));
    guide_infer_kernel<<<blocks, kInferWarps * 32, infer_smem(), st>>>(net, queries, cap, nDev, mix);
    return (int)cudaGetLastError();
}
}
}

// ------------------------------------------------------------------ host side
using namespace lfrt;
using namespace lfd::guide;

struct lf_guide
{
    lf_ctx* ctx = nullptr;
    std::vector<void*> allocs;
    float* wMaster = nullptr;
    __half* wWork = nullptr;
    float* wM = nullptr;
    float* wV = nullptr;
    float* wGrad = nullptr;
    float* gMaster = nullptr;
    __half* gWork = nullptr;
    float* gM = nullptr;
    float* gV = nullptr;
    float* gGrad = nullptr;
    float* dLoss = nullptr;
    float* scratch = nullptr;       // device samples of the host-buffer entry points
    size_t scratchFloats = 0;
    Net net{};
    int step = 0;
    float lr = 1e-2f;
    int tensorPath = 1;             // MLP on tcgen05 (1, default) or warp-level mma.sync (0)
};

namespace guidehost
{
void res_levels(int out[kLevels])
{
    const double b = std::exp((std::log(512.0) - std::log(16.0)) / (kLevels - 1));
    for (int l = 0; l < kLevels; ++l) out[l] = (int)std::floor(16.0 * std::pow(b, (double)l));
}

lf_status ensure_scratch(lf_guide* gd, size_t floats)
{
    if (gd->scratchFloats >= floats) return LF_OK;
    if (gd->scratch) cudaFree(gd->scratch);
    gd->scratch = nullptr;
    gd->scratchFloats = 0;
    cudaError_t e = cudaMalloc((void**)&gd->scratch, floats * sizeof(float));
    if (e != cudaSuccess) return cuda_fail(gd->ctx, e, "guide scratch");
    gd->scratchFloats = floats;
    return LF_OK;
}

int grid_blocks(int n, int b) { return std::min(4096, std::max(1, (n + b - 1) / b)); }

lf_status run_gradients(lf_guide* gd, const float* d_samples, int n)
{
    lf_ctx* c = gd->ctx;
    if (gd->tensorPath)
    {
        const int e = launch_train_tc(gd->net, d_samples, n, gd->wGrad, gd->gGrad, gd->dLoss, c->d_status, c->stream);
        if (e) return cuda_fail(c, (cudaError_t)e, "guide train launch");
        return LF_OK;
    }
    static bool attr = false;
    if (!attr)
    {
        cudaFuncSetAttribute(guide_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem());
        attr = true;
    }
    int sms = 1, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int tiles = (n + 15) / 16;
    const int blocks = std::max(1, std::min(sms, (tiles + kWarps - 1) / kWarps));
    guide_train_kernel<<<blocks, kWarps * 32, train_smem(), c->stream>>>(gd->net, d_samples, n, gd->wGrad, gd->gGrad,
                                                                           gd->dLoss);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "guide train launch");
    return LF_OK;
}
}

using namespace guidehost;

namespace lfrt
{
lfd::guide::Net guide_net(const lf_guide* g) { return g->net; }
int guide_tensor_path(const lf_guide* g) { return g->tensorPath; }
}

extern "C" {

lf_status lf_guide_create(lf_ctx* c, const float scene_lo[3], const float scene_hi[3], uint64_t seed, lf_guide** out)
{
    if (!c || !scene_lo || !scene_hi || !out) return LF_ERR_INVALID;
    *out = nullptr;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    lf_guide* gd = new lf_guide;
    gd->ctx = c;
    size_t bytes = 0;
    cudaError_t e = cudaSuccess;
    auto A = [&](auto** p, size_t n) {
        if (e == cudaSuccess) e = dalloc(gd->allocs, bytes, p, n);
    };
    A(&gd->wMaster, kWeights);
    A(&gd->wWork, kWeights);
    A(&gd->wM, kWeights);
    A(&gd->wV, kWeights);
    A(&gd->wGrad, kWeights);
    A(&gd->gMaster, kGridParams);
    A(&gd->gWork, kGridParams);
    A(&gd->gM, kGridParams);
    A(&gd->gV, kGridParams);
    A(&gd->gGrad, kGridParams);
    A(&gd->dLoss, 1);
    if (e != cudaSuccess)
    {
        for (void* p : gd->allocs) cudaFree(p);
        delete gd;
        return cuda_fail(c, e, "guide allocation");
    }
    // initial parameters on the host (deterministic in the seed): grid U(-1e-4, 1e-4),
    // weights U(-s, s), s = sqrt(6 / (fan_in + fan_out)), unused outputs 40..47 zero
    std::vector<float> w(kWeights), grid(kGridParams);
    uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
    auto uni = [&]() {
        st ^= st << 13;
        st ^= st >> 7;
        st ^= st << 17;
        return (float)((st >> 40) * (1.0 / 16777216.0)) * 2.f - 1.f;
    };
    for (int i = 0; i < kWeights; ++i)
    {
        const int fo = i < kW4 ? 64 : kOut;
        const float s = std::sqrt(6.f / (float)(64 + fo));
        w[i] = uni() * s;
        if (i >= kW4 && (i - kW4) / 64 >= 40) w[i] = 0.f;
    }
    for (auto& v : grid) v = uni() * 1e-4f;
    cudaMemcpyAsync(gd->wMaster, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(gd->gMaster, grid.data(), grid.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    to_half_kernel<<<grid_blocks(kWeights, 256), 256, 0, c->stream>>>(gd->wMaster, gd->wWork, kWeights);
    to_half_kernel<<<grid_blocks(kGridParams, 256), 256, 0, c->stream>>>(gd->gMaster, gd->gWork, kGridParams);
    for (float* p : {gd->wM, gd->wV, gd->wGrad}) cudaMemsetAsync(p, 0, kWeights * sizeof(float), c->stream);
    for (float* p : {gd->gM, gd->gV, gd->gGrad}) cudaMemsetAsync(p, 0, (size_t)kGridParams * sizeof(float), c->stream);
    cudaMemsetAsync(gd->dLoss, 0, sizeof(float), c->stream);
    gd->net.W = gd->wWork;
    gd->net.grid = gd->gWork;
    res_levels(gd->net.res);
    for (int a = 0; a < 3; ++a)
    {
        gd->net.lo[a] = scene_lo[a];
        const float ext = scene_hi[a] - scene_lo[a];
        gd->net.invExt[a] = ext > 0.f ? 1.f / ext : 0.f;
    }
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
    {
        for (void* p : gd->allocs) cudaFree(p);
        delete gd;
        return cuda_fail(c, e, "guide init");
    }
    *out = gd;
    return LF_OK;
}

lf_status lf_guide_release(lf_guide* gd)
{
    if (!gd) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(gd->ctx->mu);
    cudaSetDevice(gd->ctx->device);
    cudaStreamSynchronize(gd->ctx->stream);
    for (void* p : gd->allocs) cudaFree(p);
    if (gd->scratch) cudaFree(gd->scratch);
    delete gd;
    return LF_OK;
}

lf_status lf_guide_get_params(lf_guide* gd, float* weights, float* grid)
{
    if (!gd || !weights || !grid) return LF_ERR_INVALID;
    lf_ctx* c = gd->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    cudaMemcpyAsync(weights, gd->wMaster, kWeights * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(grid, gd->gMaster, (size_t)kGridParams * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? LF_OK : cuda_fail(c, e, "guide readback");
}

lf_status lf_guide_set_params(lf_guide* gd, const float* weights, const float* grid)
{
    if (!gd || !weights || !grid) return LF_ERR_INVALID;
    lf_ctx* c = gd->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    cudaMemcpyAsync(gd->wMaster, weights, kWeights * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(gd->gMaster, grid, (size_t)kGridParams * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    to_half_kernel<<<grid_blocks(kWeights, 256), 256, 0, c->stream>>>(gd->wMaster, gd->wWork, kWeights);
    to_half_kernel<<<grid_blocks(kGridParams, 256), 256, 0, c->stream>>>(gd->gMaster, gd->gWork, kGridParams);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? LF_OK : cuda_fail(c, e, "guide parameter upload");
}

lf_status lf_guide_gradients(lf_guide* gd, const float* samples, int32_t n, float* dweights, float* dgrid, float* loss)
{
    if (!gd || !samples || n <= 0 || !dweights || !dgrid || !loss) return LF_ERR_INVALID;
    lf_ctx* c = gd->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    lf_status st = ensure_scratch(gd, (size_t)n * kSampleFloats);
    if (st != LF_OK) return st;
    cudaMemcpyAsync(gd->scratch, samples, (size_t)n * kSampleFloats * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    cudaMemsetAsync(gd->wGrad, 0, kWeights * sizeof(float), c->stream);
    cudaMemsetAsync(gd->gGrad, 0, (size_t)kGridParams * sizeof(float), c->stream);
    cudaMemsetAsync(gd->dLoss, 0, sizeof(float), c->stream);
    st = run_gradients(gd, gd->scratch, n);
    if (st != LF_OK) return st;
    cudaMemcpyAsync(dweights, gd->wGrad, kWeights * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(dgrid, gd->gGrad, (size_t)kGridParams * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(loss, gd->dLoss, sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    cudaMemsetAsync(gd->wGrad, 0, kWeights * sizeof(float), c->stream);
    cudaMemsetAsync(gd->gGrad, 0, (size_t)kGridParams * sizeof(float), c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "guide gradients");
    const float inv = 1.f / (float)n;
    for (int i = 0; i < kWeights; ++i) dweights[i] *= inv;
    for (int i = 0; i < kGridParams; ++i) dgrid[i] *= inv;
    *loss *= inv;
    return check_device(c);
}

lf_status lf_guide_train_device(lf_guide* gd, const float* d_samples, int32_t n, float lr)
{
    if (!gd || !d_samples || n <= 0 || !(lr > 0.f)) return LF_ERR_INVALID;
    lf_ctx* c = gd->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    lf_status st = run_gradients(gd, d_samples, n);
    if (st != LF_OK) return st;
    ++gd->step;
    const float b1 = 0.9f, b2 = 0.99f, eps = 1e-8f;
    const float c1 = 1.f - std::pow(b1, (float)gd->step), c2 = 1.f - std::pow(b2, (float)gd->step);
    const float scale = 1.f / (float)n;
    guide_adam_kernel<<<grid_blocks(kWeights, 256), 256, 0, c->stream>>>(gd->wMaster, gd->wWork, gd->wM, gd->wV,
                                                                           gd->wGrad, kWeights, lr, b1, b2, eps, c1,
                                                                           c2, scale);
    guide_adam_kernel<<<grid_blocks(kGridParams, 256), 256, 0, c->stream>>>(gd->gMaster, gd->gWork, gd->gM, gd->gV,
                                                                              gd->gGrad, kGridParams, lr, b1, b2, eps,
                                                                              c1, c2, scale);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LF_OK : cuda_fail(c, e, "guide adam launch");
}

lf_status lf_guide_train(lf_guide* gd, const float* samples, int32_t n, float lr, float* loss)
{
    if (!gd || !samples || n <= 0) return LF_ERR_INVALID;
    lf_ctx* c = gd->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    lf_status st = ensure_scratch(gd, (size_t)n * kSampleFloats);
    if (st != LF_OK) return st;
    cudaMemcpyAsync(gd->scratch, samples, (size_t)n * kSampleFloats * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    cudaMemsetAsync(gd->dLoss, 0, sizeof(float), c->stream);
    st = lf_guide_train_device(gd, gd->scratch, n, lr);
    if (st != LF_OK) return st;
    if (loss)
    {
        cudaMemcpyAsync(loss, gd->dLoss, sizeof(float), cudaMemcpyDeviceToHost, c->stream);
        cudaStreamSynchronize(c->stream);
        *loss /= (float)n;
    }
    return check_device(c);
}

lf_status lf_guide_set_tensor_path(lf_guide* gd, int32_t tcgen05)
{
    if (!gd || tcgen05 < 0 || tcgen05 > 1) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(gd->ctx->mu);
    gd->tensorPath = tcgen05;
    return LF_OK;
}

lf_status lf_guide_eval(lf_guide* gd, const float* queries, int32_t n, float* mix, float* pdf)
{
    if (!gd || !queries || n <= 0 || (!mix && !pdf)) return LF_ERR_INVALID;
    lf_ctx* c = gd->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    const size_t qf = (size_t)n * kSampleFloats;
    lf_status st = ensure_scratch(gd, qf + (size_t)n * (kMixFloats + 1));
    if (st != LF_OK) return st;
    float* dq = gd->scratch;
    float* dmix = gd->scratch + qf;
    float* dpdf = dmix + (size_t)n * kMixFloats;
    cudaMemcpyAsync(dq, queries, qf * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    const int ie = gd->tensorPath ? launch_infer_tc(gd->net, dq, nullptr, n, dmix, c->d_status, c->stream)
                                  : launch_infer(gd->net, dq, nullptr, n, dmix, c->stream);
    if (ie) return cuda_fail(c, (cudaError_t)ie, "guide inference launch");
    guide_pdf_kernel<<<grid_blocks(n, 256), 256, 0, c->stream>>>(dmix, dq, n, dpdf);
    if (mix) cudaMemcpyAsync(mix, dmix, (size_t)n * kMixFloats * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (pdf) cudaMemcpyAsync(pdf, dpdf, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "guide eval");
    return check_device(c);
}
}
