// Guide MLP inference on the 5th-generation tensor cores (tcgen05): one CTA of 128 threads runs
// tiles of 128 queries, one query per thread, through the four layers as 128-row MMAs with the
// accumulators in tensor memory (TMEM).
//
// Per tile: every thread encodes its query (hash grid + one-blob bins, the same FP16 values as
// the warp-level kernel in lf_guide.cu) into its row of the A tile in shared memory; one thread
// issues the layer's tcgen05.mma (M = 128, N = 64 or 48, K = 64 as four K = 16 steps, FP16
// operands, FP32 accumulation) and commits it to an mbarrier; every thread then reads its own
// row of the accumulator back with tcgen05.ld (TMEM lane = query), applies ReLU, rounds to FP16
// and writes the row as the next layer's A operand. The last layer's 40 outputs become the
// query's mixture in registers. Layers alternate between two 64-column accumulators.
//
// Shared-memory operands use the canonical no-swizzle K-major layout of the MMA descriptors:
// 8 x 16-byte core matrices, stored contiguously; core matrices adjacent along K are 128 B
// apart (leading byte offset) and adjacent 8-row groups 1024 B apart (stride byte offset).
// The weights [out][in] are the B operands (N = out rows, K = in), so they are used as stored,
// re-laid into core matrices once per CTA.
//
// Every wait is bounded: an mbarrier wait that runs out sets LF_DEVERR_GUIDE_TIMEOUT in the
// status word, all threads agree on it at the next barrier, and the CTA frees its TMEM and
// returns.
#include <cuda_fp16.h>

#include <algorithm>

#include "lf_guide.cuh"
#include "lf_internal.h"

namespace lfd
{
namespace guide
{
namespace
{
constexpr int kTcRows = 128;                         // queries per tile = MMA M
constexpr int kTcThreads = 128;                      // one thread per query
constexpr uint32_t kTmemCols = 128;                  // two 64-column FP32 accumulators
constexpr int kTileBytes = kTcRows * kIn * 2;        // A tile: 128 x 64 FP16
constexpr int kLayerBytes = 64 * 64 * 2;             // W1..W3: 64 x 64 FP16
constexpr int kWBytes = 3 * kLayerBytes + kOut * 64 * 2;
constexpr int kTcSmem = kWBytes + kTileBytes + 16;   // + mbarrier and TMEM address
constexpr uint32_t kLbo = 128;                       // core matrices adjacent along K
constexpr uint32_t kSbo = 1024;                      // adjacent 8-row groups (8 core matrices of K = 64)
constexpr long long kWaitCycles = 4000000000LL;      // ~2 s at 2 GHz

// Byte offset of element (row, k) of a K = 64 operand in the canonical no-swizzle layout.
__device__ __forceinline__ uint32_t cm_offset(int row, int k)
{
    return (uint32_t)(((row >> 3) * 8 + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05): start address, leading and stride byte offsets
// (all >> 4), descriptor version 1 (bits 46-47), base offset 0, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((kLbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((kSbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B FP16 (bits 7-9, 10-12 =
// 0), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N)
{
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Bounded wait for the mbarrier phase with parity `phase`; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase)
{
    const long long t0 = clock64();
    while (true)
    {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(mbar), "r"(phase)
            : "memory");
        if (ok) return true;
        if (clock64() - t0 > kWaitCycles) return false;
    }
}

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void store8(unsigned char* tile, int row, int k0, const float* v)
{
    __half2 h[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) h[i] = __floats2half2_rn(v[2 * i], v[2 * i + 1]);
    *reinterpret_cast<uint4*>(tile + cm_offset(row, k0)) = *reinterpret_cast<const uint4*>(h);
}

// The query's 64 input features (same values and FP16 rounding as encode_tile in lf_guide.cu)
// into its row of the A tile.
__device__ __forceinline__ void encode_row(const Net& net, const float* rec, bool valid, unsigned char* tile, int row)
{
    float f[64];
    if (!valid)
    {
#pragma unroll
        for (int i = 0; i < 64; ++i) f[i] = 0.f;
    }
    else
    {
        float p01[3];
        position01(net, rec, p01);
#pragma unroll 1
        for (int l = 0; l < kLevels; ++l)
        {
            uint32_t idx[8];
            float w[8];
            grid_corners(net.res[l], p01, idx, w);
            const __half* tab = net.grid + (size_t)l * kT * kFeatures;
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            for (int c = 0; c < 8; ++c)
            {
                const uint2 v = *reinterpret_cast<const uint2*>(tab + (size_t)idx[c] * kFeatures);
                const __half2 a = *reinterpret_cast<const __half2*>(&v.x), b = *reinterpret_cast<const __half2*>(&v.y);
                acc[0] += w[c] * __low2float(a);
                acc[1] += w[c] * __high2float(a);
                acc[2] += w[c] * __low2float(b);
                acc[3] += w[c] * __high2float(b);
            }
            // unrolled stores keep f[] in registers
#pragma unroll
            for (int q = 0; q < kLevels; ++q)
                if (q == l)
                {
                    f[4 * q + 0] = acc[0];
                    f[4 * q + 1] = acc[1];
                    f[4 * q + 2] = acc[2];
                    f[4 * q + 3] = acc[3];
                }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h)
        {
            const float* d = rec + 3 + 3 * h;   // outgoing direction, then the normal
            float th, ph;
            sph01(d[0], d[1], d[2], &th, &ph);
#pragma unroll
            for (int k = 0; k < kBlobBins; ++k)
            {
                f[32 + h * 16 + k] = blob(th, k);
                f[32 + h * 16 + 8 + k] = blob(ph, k);
            }
        }
    }
#pragma unroll
    for (int k0 = 0; k0 < 64; k0 += 8) store8(tile, row, k0, f + k0);
}
}

__global__ void __launch_bounds__(kTcThreads, 1)
    guide_infer_tc_kernel(Net net, const float* queries, int n, const int* nDev, float* mix, uint32_t* status)
{
    if (nDev) n = *nDev;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sW = smem;
    unsigned char* sA = smem + kWBytes;
    uint64_t* mbarPtr = reinterpret_cast<uint64_t*>(smem + kWBytes + kTileBytes);
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(smem + kWBytes + kTileBytes + 8);
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t mbar = smem_addr(mbarPtr);

    // weights [out][in] of the four layers -> B operands in core-matrix layout
    for (int i = tid; i < kWeights; i += kTcThreads)
    {
        const int l = i < 3 * 4096 ? i >> 12 : 3;
        const int r = (i - l * 4096) >> 6, k = (i - l * 4096) & 63;
        *reinterpret_cast<__half*>(sW + l * kLayerBytes + cm_offset(r, k)) = net.W[i];
    }
    if (warp == 0)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmemSlot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmemSlot;
    const uint32_t lane0 = (uint32_t)(warp * 32) << 16;   // this warp's TMEM lane quarter
    const uint32_t aBase = smem_addr(sA), wBase = smem_addr(sW);
    uint32_t phase = 0;
    bool failed = false;

    const int tiles = (n + kTcRows - 1) / kTcRows;
    for (int tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x)
    {
        const int q = tile * kTcRows + tid;
        const bool valid = q < n;
        encode_row(net, queries + (size_t)(valid ? q : 0) * kSampleFloats, valid, sA, tid);
        float out[48];
        for (int layer = 0; layer < 4; ++layer)
        {
            fence_async_smem();
            fence_before_sync();
            __syncthreads();
            const uint32_t dcol = (uint32_t)(layer & 1) * 64u;
            if (tid == 0)
            {
                fence_after_sync();
                const uint32_t idesc = instr_desc(kTcRows, layer < 3 ? 64 : kOut);
#pragma unroll
                for (int s = 0; s < 4; ++s)
                    mma_f16(tmem + dcol, smem_desc(aBase + s * 256), smem_desc(wBase + layer * kLayerBytes + s * 256),
                            idesc, s > 0 ? 1u : 0u);
                mma_commit(mbar);
            }
            const bool ok = mbar_wait(mbar, phase);
            phase ^= 1u;
            if (__syncthreads_or(!ok))
            {
                if (tid == 0) atomicOr(status, LF_DEVERR_GUIDE_TIMEOUT);
                failed = true;
                break;
            }
            fence_after_sync();
            if (layer < 3)
            {
#pragma unroll
                for (int c = 0; c < 64; c += 16)
                {
                    float v[16];
                    tmem_ld16(tmem + lane0 + dcol + c, v);
                    tmem_wait_ld();
#pragma unroll
                    for (int i = 0; i < 16; ++i) v[i] = fmaxf(v[i], 0.f);
                    store8(sA, tid, c, v);
                    store8(sA, tid, c + 8, v + 8);
                }
            }
            else
            {
#pragma unroll
                for (int c = 0; c < kOut; c += 16) tmem_ld16(tmem + lane0 + dcol + c, out + c);
                tmem_wait_ld();
            }
        }
        if (failed) break;
        if (valid)
        {
            float* dst = mix + (size_t)q * kMixFloats;
            float mx = -1e30f;
            for (int i = 0; i < kLobes; ++i) mx = fmaxf(mx, out[5 * i + 4]);
            float es = 0.f, e[kLobes];
            for (int i = 0; i < kLobes; ++i)
            {
                e[i] = __expf(out[5 * i + 4] - mx);
                es += e[i];
            }
            float cum = 0.f;
            for (int i = 0; i < kLobes; ++i)
            {
                float mu[3], k;
                lobe_params(out + 5 * i, mu, &k);
                cum += e[i] / es;
                dst[5 * i + 0] = mu[0];
                dst[5 * i + 1] = mu[1];
                dst[5 * i + 2] = mu[2];
                dst[5 * i + 3] = k;
                dst[5 * i + 4] = i == kLobes - 1 ? 1.f : cum;
            }
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0)
    {
        fence_after_sync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

int launch_infer_tc(const Net& net, const float* queries, const int* nDev, int cap, float* mix, uint32_t* status,
                    cudaStream_t st)
{
    static bool attr = false;
    if (!attr)
    {
        cudaFuncSetAttribute(guide_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
        attr = true;
    }
    int sms = 1, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // at most 4 CTAs per SM: 4 x 128 TMEM columns fill the SM's 512, so no allocation waits
    const int perSm = std::min(4, occupancy_blocks_per_sm((const void*)guide_infer_tc_kernel, kTcThreads, kTcSmem));
    const int tiles = (cap + kTcRows - 1) / kTcRows;
    const int blocks = std::max(1, std::min(sms * std::max(1, perSm), tiles));
    guide_infer_tc_kernel<<<blocks, kTcThreads, kTcSmem, st>>>(net, queries, cap, nDev, mix, status);
    return (int)cudaGetLastError();
}
}
}
