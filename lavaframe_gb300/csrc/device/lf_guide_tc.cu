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
// Training (guide_train_tc_kernel) runs the same forward pass with every activation tile kept
// in shared memory, then the backward pass layer by layer: the output gradient dY (one row per
// sample, FP16) times W^T gives the previous layer's gradient (M = 128 samples, K = out), and
// the weight gradient dW[out][in] += dY^T H sums over the tile's 128 samples as the MMA's K
// dimension. For that product the row-per-sample tiles dY [s][out] and H [s][in] are read
// MN-major (the transpose bits of the instruction descriptor): their 16-byte chunks run along
// out and in, which for dW are the M and N dimensions. dY is kept 128 columns wide with zeros
// beyond the layer's outputs, so dW is a 128-row MMA whose rows 0..63 are the layer's. The
// four dW accumulators stay in TMEM across every tile the CTA processes and are added to the
// global gradient once at the end; the grid-feature gradients are scattered with the
// trilinear weights per sample, as in the warp-level kernel.
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
constexpr int kTcThreads = 128;                      // one thread per query (training)
constexpr int kTileBytes = kTcRows * kIn * 2;        // A tile: 128 x 64 FP16
constexpr int kLayerBytes = 64 * 64 * 2;             // W1..W3: 64 x 64 FP16
constexpr int kWBytes = 3 * kLayerBytes + kOut * 64 * 2;
// Inference: kInferGroups warpgroups per CTA, each running its own tiles through its own A tile,
// 64 TMEM columns and mbarrier; the weights in shared memory are the CTA's, shared.
constexpr int kInferGroups = 2;
constexpr int kInferThreads = 128 * kInferGroups;
constexpr int kInferCtasPerSm = 3;                   // 3 x 64 KB shared memory, 3 x 128 TMEM columns
constexpr uint32_t kTmemCols = 64 * kInferGroups;
constexpr int kTcSmem = kWBytes + kInferGroups * kTileBytes + 16 * kInferGroups;   // + per group mbarrier, TMEM address
constexpr uint32_t kLbo = 128;                       // core matrices adjacent along K
constexpr uint32_t kSbo = 1024;                      // adjacent 8-row groups (8 core matrices of K = 64)
constexpr long long kWaitCycles = 4000000000LL;      // ~2 s at 2 GHz

// Byte offset of element (row, k) of an operand with kg core matrices along K (K = 8 kg) in
// the canonical no-swizzle layout: core matrix (row / 8, k / 8) at ((row / 8) kg + k / 8) x 128.
__device__ __forceinline__ uint32_t cm_offset(int row, int k, int kg = 8)
{
    return (uint32_t)(((row >> 3) * kg + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05): start address, leading byte offset (between
// core matrices adjacent along K) and stride byte offset (between core matrices adjacent along
// M or N), all >> 4; descriptor version 1 (bits 46-47), base offset 0, no swizzle (bits 61-63).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo = kLbo, uint32_t sbo = kSbo)
{
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B FP16 (bits 7-9, 10-12 =
// 0), A and B K-major (bits 15, 16 = 0) or MN-major (1), N >> 3 at bits 17-22, M >> 4 at
// bits 24-28.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N, bool aMN = false, bool bMN = false)
{
    return (1u << 4) | ((aMN ? 1u : 0u) << 15) | ((bMN ? 1u : 0u) << 16) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
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

// One FP32 accumulator column of this thread's TMEM lane.
__device__ __forceinline__ float tmem_ld1(uint32_t taddr)
{
    uint32_t r;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(r) : "r"(taddr));
    return __uint_as_float(r);
}

__device__ __forceinline__ void store8(unsigned char* tile, int row, int k0, const float* v, int kg = 8)
{
    __half2 h[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) h[i] = __floats2half2_rn(v[2 * i], v[2 * i + 1]);
    *reinterpret_cast<uint4*>(tile + cm_offset(row, k0, kg)) = *reinterpret_cast<const uint4*>(h);
}

// 8 FP16 values of a row (16 bytes) as floats.
__device__ __forceinline__ void load8(const unsigned char* tile, int row, int k0, float* v, int kg = 8)
{
    const uint4 q = *reinterpret_cast<const uint4*>(tile + cm_offset(row, k0, kg));
    const __half2* h = reinterpret_cast<const __half2*>(&q);
#pragma unroll
    for (int i = 0; i < 4; ++i)
    {
        v[2 * i] = __low2float(h[i]);
        v[2 * i + 1] = __high2float(h[i]);
    }
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
            float acc[4];
            level_features(net, l, p01, acc);
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

// Inference form of encode_row: the same FP16 values, written level by level (8 bytes at a
// time) so that no 64-feature array stays live.
__device__ __forceinline__ void encode_row_direct(const Net& net, const float* rec, bool valid, unsigned char* tile,
                                                  int row)
{
    if (!valid)
    {
#pragma unroll
        for (int k0 = 0; k0 < 64; k0 += 8) *reinterpret_cast<uint4*>(tile + cm_offset(row, k0)) = make_uint4(0, 0, 0, 0);
        return;
    }
    float p01[3];
    position01(net, rec, p01);
#pragma unroll 1
    for (int l = 0; l < kLevels; ++l)
    {
        float acc[4];
        level_features(net, l, p01, acc);
        const __half2 h0 = __floats2half2_rn(acc[0], acc[1]), h1 = __floats2half2_rn(acc[2], acc[3]);
        uint2 o;
        o.x = *reinterpret_cast<const uint32_t*>(&h0);
        o.y = *reinterpret_cast<const uint32_t*>(&h1);
        *reinterpret_cast<uint2*>(tile + cm_offset(row, 4 * l)) = o;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
    {
        const float* d = rec + 3 + 3 * h;   // outgoing direction, then the normal
        float th, ph;
        sph01(d[0], d[1], d[2], &th, &ph);
        float f[8];
#pragma unroll
        for (int k = 0; k < kBlobBins; ++k) f[k] = blob(th, k);
        store8(tile, row, 32 + h * 16, f);
#pragma unroll
        for (int k = 0; k < kBlobBins; ++k) f[k] = blob(ph, k);
        store8(tile, row, 32 + h * 16 + 8, f);
    }
}

// Barrier of one warpgroup (named barrier id, 128 threads).
__device__ __forceinline__ void group_sync(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }

// Barrier of one warpgroup that returns whether any of its threads passed true.
__device__ __forceinline__ bool group_sync_or(int id, bool v)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, %2, 128, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id)
        : "memory");
    return r != 0;
}
}

// kInferGroups warpgroups per CTA; warpgroup g takes tiles blockIdx.x * kInferGroups + g,
// stepping by gridDim.x * kInferGroups, and synchronises on its own named barrier (1 + g), so
// that one group's MMAs and waits overlap the other's encoding and epilogue.
__global__ void __launch_bounds__(kInferThreads, kInferCtasPerSm)
    guide_infer_tc_kernel(Net net, const float* queries, int n, const int* nDev, float* mix, uint32_t* status)
{
    if (nDev) n = *nDev;
    extern __shared__ __align__(1024) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int grp = tid >> 7, row = tid & 127;
    unsigned char* sW = smem;
    unsigned char* sA = smem + kWBytes + grp * kTileBytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kWBytes + kInferGroups * kTileBytes);
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(bars + kInferGroups);
    const uint32_t mbar = smem_addr(bars + grp);

    // weights [out][in] of the four layers -> B operands in core-matrix layout
    for (int i = tid; i < kWeights; i += kInferThreads)
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
    if (row == 0)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    // the group's 64 accumulator columns; warp w reads TMEM lanes 32 (w % 4) .. + 31
    const uint32_t acc = *tmemSlot + (uint32_t)(64 * grp);
    const uint32_t lane0 = (uint32_t)((warp & 3) * 32) << 16;
    const uint32_t aBase = smem_addr(sA), wBase = smem_addr(sW);
    const int barId = 1 + grp;
    uint32_t phase = 0;
    bool failed = false;

    const int tiles = (n + kTcRows - 1) / kTcRows;
    for (int tile = blockIdx.x * kInferGroups + grp; tile < tiles && !failed; tile += gridDim.x * kInferGroups)
    {
        const int q = tile * kTcRows + row;
        const bool valid = q < n;
        encode_row_direct(net, queries + (size_t)(valid ? q : 0) * kSampleFloats, valid, sA, row);
        for (int layer = 0; layer < 4; ++layer)
        {
            // the group's A tile (and, from layer 1, its reads of the accumulator) are complete
            fence_async_smem();
            fence_before_sync();
            group_sync(barId);
            if (row == 0)
            {
                fence_after_sync();
                const uint32_t idesc = instr_desc(kTcRows, layer < 3 ? 64 : kOut);
#pragma unroll
                for (int s = 0; s < 4; ++s)
                    mma_f16(acc, smem_desc(aBase + s * 256), smem_desc(wBase + layer * kLayerBytes + s * 256), idesc,
                            s > 0 ? 1u : 0u);
                mma_commit(mbar);
            }
            const bool ok = mbar_wait(mbar, phase);
            phase ^= 1u;
            if (group_sync_or(barId, !ok))
            {
                if (row == 0) atomicOr(status, LF_DEVERR_GUIDE_TIMEOUT);
                failed = true;
                break;
            }
            fence_after_sync();
            if (layer == 3) break;   // the outputs stay in TMEM for the epilogue
#pragma unroll
            for (int c = 0; c < 64; c += 16)
            {
                float v[16];
                tmem_ld16(acc + lane0 + c, v);
                tmem_wait_ld();
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = fmaxf(v[i], 0.f);
                store8(sA, row, c, v);
                store8(sA, row, c + 8, v + 8);
            }
        }
        if (failed) break;
        // epilogue straight from the accumulator: the eight logits first (softmax), then lobe
        // by lobe its mean and concentration, so that few outputs are live at a time; the TMEM
        // loads are warp-wide, the stores for valid queries only
        float e[kLobes];
#pragma unroll
        for (int i = 0; i < kLobes; ++i) e[i] = tmem_ld1(acc + lane0 + 5 * i + 4);
        tmem_wait_ld();
        float mx = -1e30f;
#pragma unroll
        for (int i = 0; i < kLobes; ++i) mx = fmaxf(mx, e[i]);
        float es = 0.f;
#pragma unroll
        for (int i = 0; i < kLobes; ++i)
        {
            e[i] = __expf(e[i] - mx);
            es += e[i];
        }
        const float invEs = 1.f / es;
        float* dst = mix + (size_t)(valid ? q : 0) * kMixFloats;
        float cum = 0.f;
#pragma unroll
        for (int i = 0; i < kLobes; ++i)
        {
            float o5[4], mu[3], k;
#pragma unroll
            for (int j = 0; j < 4; ++j) o5[j] = tmem_ld1(acc + lane0 + 5 * i + j);
            tmem_wait_ld();
            lobe_params(o5, mu, &k);
            cum += e[i] * invEs;
            if (valid)
            {
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
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(*tmemSlot), "r"(kTmemCols)
                     : "memory");
    }
}

namespace
{
// Shared memory of the training kernel, in this order so that every operand's span lies well
// inside the allocation: dY (128 samples x 128 outputs, columns beyond the layer's outputs
// zero), the input tile X and the activation tiles H1..H3 (128 x 64 each), the weights as
// forward B operands [out][in] and as backward B operands W^T [in][out], then the mbarrier and
// the TMEM address.
constexpr int kDyBytes = 128 * 128 * 2;
constexpr int kOffDy = 0;
constexpr int kOffX = kOffDy + kDyBytes;
constexpr int kOffH = kOffX + kTileBytes;                 // H1, H2, H3
constexpr int kOffW = kOffH + 3 * kTileBytes;
constexpr int kOffWT = kOffW + kWBytes;
constexpr int kOffBar = kOffWT + kWBytes;
constexpr int kTrainSmem = kOffBar + 16;
constexpr uint32_t kTrainTmemCols = 512;                  // 2 x 64 forward/backward + 4 x 64 dW
constexpr uint32_t kColDW = 128;                          // dW of layer l at kColDW + 64 l
constexpr int kDyKg = 16;                                 // dY: 16 core matrices along its 128 columns

// Issues one MMA group (k steps of K = 16) and commits it to the mbarrier; thread 0 only.
__device__ __forceinline__ void issue(uint32_t dtmem, uint32_t a, uint32_t aStep, uint32_t aLbo, uint32_t aSbo, uint32_t b,
                                      uint32_t bStep, uint32_t bLbo, uint32_t bSbo, uint32_t idesc, int steps, bool acc)
{
    for (int k = 0; k < steps; ++k)
        mma_f16(dtmem, smem_desc(a + k * aStep, aLbo, aSbo), smem_desc(b + k * bStep, bLbo, bSbo), idesc,
                (acc || k > 0) ? 1u : 0u);
}
}

// One pass over n training samples: adds the per-sample gradients (not divided by n) of every
// weight into gW and of every grid parameter into gGrid, and the summed loss into loss - the
// same sums as guide_train_kernel, with the products on tcgen05.
__global__ void __launch_bounds__(kTcThreads, 1)
    guide_train_tc_kernel(Net net, const float* samples, int n, float* gW, float* gGrid, float* loss,
                          uint32_t* status)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sDy = smem + kOffDy;
    unsigned char* sX = smem + kOffX;
    unsigned char* sH = smem + kOffH;
    unsigned char* sW = smem + kOffW;
    unsigned char* sWT = smem + kOffWT;
    uint64_t* mbarPtr = reinterpret_cast<uint64_t*>(smem + kOffBar);
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(smem + kOffBar + 8);
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t mbar = smem_addr(mbarPtr);

    // weights: forward B operands [out][in] (K = in) and backward B operands [in][out]
    // (K = out: 8 core matrices for W1..W3, 6 for W4)
    for (int i = tid; i < kWeights; i += kTcThreads)
    {
        const int l = i < 3 * 4096 ? i >> 12 : 3;
        const int o = (i - l * 4096) >> 6, k = (i - l * 4096) & 63;
        const __half w = net.W[i];
        *reinterpret_cast<__half*>(sW + l * kLayerBytes + cm_offset(o, k)) = w;
        *reinterpret_cast<__half*>(sWT + l * kLayerBytes + cm_offset(k, o, l < 3 ? 8 : 6)) = w;
    }
    // dY columns 64..127 stay zero (the padding rows of the dW products)
    for (int i = tid; i < kDyBytes / 16; i += kTcThreads) reinterpret_cast<uint4*>(sDy)[i] = make_uint4(0, 0, 0, 0);
    if (warp == 0)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmemSlot)),
                     "r"(kTrainTmemCols)
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
    const uint32_t lane0 = (uint32_t)(warp * 32) << 16;
    const uint32_t aDy = smem_addr(sDy), aX = smem_addr(sX), aH = smem_addr(sH), aW = smem_addr(sW),
                   aWT = smem_addr(sWT);
    uint32_t phase = 0;
    bool failed = false, any = false;
    float lossSum = 0.f;

    // one MMA group per call site: sync the operands written by all threads, issue, wait
    auto run = [&](auto&& issueFn) -> bool {
        fence_async_smem();
        fence_before_sync();
        __syncthreads();
        if (tid == 0)
        {
            fence_after_sync();
            issueFn();
            mma_commit(mbar);
        }
        const bool ok = mbar_wait(mbar, phase);
        phase ^= 1u;
        if (__syncthreads_or(!ok))
        {
            if (tid == 0) atomicOr(status, LF_DEVERR_GUIDE_TIMEOUT);
            return false;
        }
        fence_after_sync();
        return true;
    };

    const uint32_t idFwd = instr_desc(kTcRows, 64), idOut = instr_desc(kTcRows, kOut);
    const uint32_t idDw = instr_desc(128, 64, true, true);
    const int tiles = (n + kTcRows - 1) / kTcRows;
    for (int tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x)
    {
        const int q = tile * kTcRows + tid;
        const bool valid = q < n;
        const float* rec = samples + (size_t)(valid ? q : 0) * kSampleFloats;
        encode_row(net, rec, valid, sX, tid);
        // forward: H1..H3 = relu(A W^T) into their tiles, outputs into registers
        float out[48];
        for (int layer = 0; layer < 4 && !failed; ++layer)
        {
            const uint32_t a = layer == 0 ? aX : aH + (layer - 1) * kTileBytes;
            const uint32_t dcol = (uint32_t)(layer & 1) * 64u;
            failed = !run([&] { issue(tmem + dcol, a, 256, kLbo, kSbo, aW + layer * kLayerBytes, 256, kLbo, kSbo,
                                      layer < 3 ? idFwd : idOut, 4, false); });
            if (failed) break;
            if (layer < 3)
            {
                unsigned char* h = sH + layer * kTileBytes;
#pragma unroll
                for (int c = 0; c < 64; c += 16)
                {
                    float v[16];
                    tmem_ld16(tmem + lane0 + dcol + c, v);
                    tmem_wait_ld();
#pragma unroll
                    for (int i = 0; i < 16; ++i) v[i] = fmaxf(v[i], 0.f);
                    store8(h, tid, c, v);
                    store8(h, tid, c + 8, v + 8);
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
        // loss and the output gradient (40 used of 48; columns 40..63 zero)
        {
            float d[64];
#pragma unroll
            for (int k = 0; k < 64; ++k) d[k] = 0.f;
            if (valid) lossSum += sample_loss_grad(out, rec + 9, rec[12], d);
#pragma unroll
            for (int k0 = 0; k0 < 64; k0 += 8) store8(sDy, tid, k0, d + k0, kDyKg);
        }
        // backward, layer 4 .. 1: dH = dY W (into the free forward column half) and
        // dW += dY^T H (accumulated across tiles); then dY of the layer below = dH * relu'(H)
        for (int layer = 3; layer >= 0 && !failed; --layer)
        {
            const uint32_t dcol = (uint32_t)(layer & 1) * 64u;
            const uint32_t hIn = layer == 0 ? aX : aH + (layer - 1) * kTileBytes;   // this layer's input
            const int kSteps = layer == 3 ? 3 : 4;                                   // K = 48 or 64 outputs
            const int nIn = layer == 0 ? 32 : 64;                                    // input gradients needed
            const bool accW = any;
            failed = !run([&] {
                // dH[s][in] = sum_out dY[s][out] W[out][in]: A = dY (K-major, K = out), B = W^T
                issue(tmem + dcol, aDy, 256, kLbo, kDyKg * 128, aWT + layer * kLayerBytes, 256, kLbo,
                      (layer < 3 ? 8 : 6) * 128, instr_desc(kTcRows, nIn), kSteps, false);
                // dW[out][in] += sum_s dY[s][out] H[s][in]: A = dY^T (MN-major, M = 128 padded
                // outputs), B = H^T (MN-major, N = 64 inputs); K = the tile's 128 samples
                issue(tmem + kColDW + 64 * layer, aDy, 2 * kDyKg * 128, kDyKg * 128, 128, hIn, 2 * 1024, 1024, 128,
                      idDw, 8, accW);
            });
            if (failed) break;
            if (layer > 0)
            {
                // dY of layer - 1 = dH masked by the ReLU of H_layer (its FP16 activations > 0)
                const unsigned char* h = sH + (layer - 1) * kTileBytes;
#pragma unroll
                for (int c = 0; c < 64; c += 16)
                {
                    float v[16], hv[16];
                    tmem_ld16(tmem + lane0 + dcol + c, v);
                    tmem_wait_ld();
                    load8(h, tid, c, hv);
                    load8(h, tid, c + 8, hv + 8);
#pragma unroll
                    for (int i = 0; i < 16; ++i) v[i] = hv[i] > 0.f ? v[i] : 0.f;
                    store8(sDy, tid, c, v, kDyKg);
                    store8(sDy, tid, c + 8, v + 8, kDyKg);
                }
            }
            else
            {
                // grid-feature gradients (inputs 0..31) scattered with the trilinear weights; the
                // warp-wide TMEM loads run on every lane, the scatter on valid samples only
                float dx[32];
#pragma unroll
                for (int c = 0; c < 32; c += 16) tmem_ld16(tmem + lane0 + dcol + c, dx + c);
                tmem_wait_ld();
                float p01[3];
                position01(net, rec, p01);
#pragma unroll 1
                for (int l = 0; l < (valid ? kLevels : 0); ++l)
                {
                    uint32_t idx[8];
                    float w[8];
                    grid_corners(net.res[l], p01, idx, w);
                    float* gt = gGrid + (size_t)l * kT * kFeatures;
                    float g4[4];
#pragma unroll
                    for (int f = 0; f < 4; ++f)
                    {
                        g4[f] = dx[0];
#pragma unroll
                        for (int qq = 0; qq < 32; ++qq)
                            if (qq == l * 4 + f) g4[f] = dx[qq];
                    }
                    for (int c = 0; c < 8; ++c)
                        for (int f = 0; f < 4; ++f) atomicAdd(&gt[(size_t)idx[c] * kFeatures + f], w[c] * g4[f]);
                }
            }
        }
        any = true;
    }
    // loss: block sum, one atomic
    for (int off = 16; off > 0; off >>= 1) lossSum += __shfl_xor_sync(0xffffffffu, lossSum, off);
    if ((tid & 31) == 0 && lossSum != 0.f) atomicAdd(loss, lossSum);
    // weight gradients: TMEM lanes 0..63 = outputs, 64 columns = inputs, one atomic each
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (!failed && any && warp < 2)
    {
        for (int layer = 0; layer < 4; ++layer)
        {
            const int o = tid;   // lanes 0..63: warps 0 and 1
            const int outs = layer < 3 ? 64 : kOut;
            const int base = layer * 4096;
            for (int c = 0; c < 64; c += 16)
            {
                float v[16];
                tmem_ld16(tmem + lane0 + kColDW + 64 * layer + c, v);
                tmem_wait_ld();
                if (o < outs)
                    for (int i = 0; i < 16; ++i)
                        if (v[i] != 0.f) atomicAdd(&gW[base + o * 64 + c + i], v[i]);
            }
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0)
    {
        fence_after_sync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTrainTmemCols)
                     : "memory");
    }
}

int launch_train_tc(const Net& net, const float* samples, int n, float* gW, float* gGrid, float* loss, uint32_t* status,
                    cudaStream_t st)
{
    static bool attr = false;
    if (!attr)
    {
        cudaFuncSetAttribute(guide_train_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmem);
        attr = true;
    }
    int sms = 1, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // one CTA per SM: its 512 TMEM columns are the SM's
    const int tiles = (n + kTcRows - 1) / kTcRows;
    const int blocks = std::max(1, std::min(sms, tiles));
    guide_train_tc_kernel<<<blocks, kTcThreads, kTrainSmem, st>>>(net, samples, n, gW, gGrid, loss, status);
    return (int)cudaGetLastError();
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
    // kInferCtasPerSm CTAs per SM: the launch bounds cap the registers for that many, shared
    // memory (about 63 KB per CTA) fits them, and their 3 x 128 TMEM columns stay within the
    // SM's 512, so no allocation waits
    const int tiles = (cap + kTcRows - 1) / kTcRows;
    const int blocks = std::max(1, std::min(sms * kInferCtasPerSm, (tiles + kInferGroups - 1) / kInferGroups));
    guide_infer_tc_kernel<<<blocks, kInferThreads, kTcSmem, st>>>(net, queries, cap, nDev, mix, status);
    return (int)cudaGetLastError();
}
}
}
