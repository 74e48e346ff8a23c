// Batched ray queries (ClosestHit / AnyHit as a service): ray binning and a persistent
// traversal kernel.
//
// Random rays give each lane of a warp its own path through the BVH: few lanes share an
// instruction and almost every node comes from DRAM. Two measures, neither of which changes
// any per-ray result:
//  - binning: rays are counting-sorted by a key made of the Morton code of their origin
//    cell (64^3 cells over the scene box; 16^3 and 32^3 measured 3 % and 1.3 % slower on the
//    microbench) and their direction octant, so neighbouring lanes start in the same region
//    heading the same way and share nodes in L1/L2;
//  - persistent warps with dynamic fetch: warps take rays 32 at a time from a counter in the
//    binned order, so a warp that finished early takes more work.
#include "lf_kernels.h"

namespace lfd
{
namespace
{
constexpr unsigned kFullMask = 0xffffffffu;
#ifndef LF_TRACE_CELL_BITS
#define LF_TRACE_CELL_BITS 6
#endif
constexpr int kCellBits = LF_TRACE_CELL_BITS;          // cells per axis = 2^kCellBits
constexpr int kCells = 1 << kCellBits;
constexpr int kBinBits = 3 * kCellBits + 3;            // origin Morton code + direction octant
constexpr int kBins = 1 << kBinBits;
constexpr int kScanBlock = 1024;
constexpr int kScanBlocks = kBins / kScanBlock;        // partial sums of the bin scan
static_assert(kScanBlocks >= 1 && kScanBlocks <= 2 * kScanBlock, "bin scan covers 2^10 to 2^21 bins");

__device__ __forceinline__ uint32_t spread3(uint32_t x)   // up to 7 bits -> every third bit
{
    x &= (uint32_t)(kCells - 1);
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

__device__ __forceinline__ uint32_t cell(float v, float lo, float inv)
{
    float q = (v - lo) * inv;
    const float top = (float)(kCells - 1);
    q = q < 0.f ? 0.f : (q > top ? top : q);
    return (uint32_t)q;
}

// Exclusive scan of 1024 values held one per thread (a block of 1024 threads): returns the
// thread's exclusive prefix and stores the block total in *total (shared memory).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total)
{
    __shared__ uint32_t warpSums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int k = 1; k < 32; k <<= 1)
    {
        const uint32_t u = __shfl_up_sync(kFullMask, incl, k);
        if (lane >= k) incl += u;
    }
    if (lane == 31) warpSums[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        const uint32_t w = warpSums[lane];
        uint32_t wi = w;
#pragma unroll
        for (int k = 1; k < 32; k <<= 1)
        {
            const uint32_t u = __shfl_up_sync(kFullMask, wi, k);
            if (lane >= k) wi += u;
        }
        warpSums[lane] = wi - w;
        if (lane == 31) *total = wi;
    }
    __syncthreads();
    return warpSums[warp] + incl - v;
}
}

__global__ void ray_keys_kernel(const float4* rays, long long n, float3 lo, float3 inv, uint32_t* keys, uint32_t* hist)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    {
        float4 o = rays[2 * i], d = rays[2 * i + 1];
        uint32_t m = (spread3(cell(o.x, lo.x, inv.x)) << 2) | (spread3(cell(o.y, lo.y, inv.y)) << 1) |
                     spread3(cell(o.z, lo.z, inv.z));
        uint32_t oct = (d.x < 0.f ? 4u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 1u : 0u);
        uint32_t k = (m << 3) | oct;
        keys[i] = k;
        atomicAdd(&hist[k], 1u);
    }
}

// Exclusive scan of the kBins counters in three launches: each block of 1024 scans its slice
// and records the slice total (hist[kBins + block]); one block scans the totals (at most two
// per thread); each block then adds its slice's offset.
__global__ void __launch_bounds__(kScanBlock) bins_scan_kernel(uint32_t* hist)
{
    __shared__ uint32_t total;
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const uint32_t v = hist[i];
    const uint32_t ex = block_exclusive_scan(v, &total);
    hist[i] = ex;
    __syncthreads();
    if (threadIdx.x == 0) hist[kBins + blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanBlock) bins_scan_totals_kernel(uint32_t* hist)
{
    __shared__ uint32_t total;
    uint32_t* sums = hist + kBins;
    const int t = threadIdx.x;
    const uint32_t a = 2 * t < kScanBlocks ? sums[2 * t] : 0u;
    const uint32_t b = 2 * t + 1 < kScanBlocks ? sums[2 * t + 1] : 0u;
    const uint32_t ex = block_exclusive_scan(a + b, &total);
    __syncthreads();
    if (2 * t < kScanBlocks) sums[2 * t] = ex;
    if (2 * t + 1 < kScanBlocks) sums[2 * t + 1] = ex + a;
}

__global__ void __launch_bounds__(kScanBlock) bins_scan_add_kernel(uint32_t* hist)
{
    hist[blockIdx.x * kScanBlock + threadIdx.x] += hist[kBins + blockIdx.x];
}

__global__ void ray_scatter_kernel(const uint32_t* keys, long long n, uint32_t* cursor, int* perm)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    {
        uint32_t pos = atomicAdd(&cursor[keys[i]], 1u);
        perm[pos] = (int)i;
    }
}

// Persistent closest-hit / any-hit over `n` rays taken in `perm` order (or input order).
template <bool kAny>
__global__ void __launch_bounds__(128) trace_persistent_kernel(DevScene S, const float4* rays, const int* perm,
                                                                long long n, int4* hits, uint8_t* occluded, int lights,
                                                                unsigned long long* next, uint32_t* status)
{
    TravState s;
    long long rid = -1;   // -1: needs a ray, -2: no rays left
    int light = -1;
    const int lane = threadIdx.x & 31;
    while (true)
    {
        unsigned need = __ballot_sync(kFullMask, rid == -1);
        if (need)
        {
            int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(next, (unsigned long long)__popc(need));
            base = __shfl_sync(kFullMask, base, leader);
            if (rid == -1)
            {
                unsigned long long my = base + __popc(need & ((1u << lane) - 1u));
                if (my < (unsigned long long)n)
                {
                    rid = perm ? (long long)perm[my] : (long long)my;
                    float4 o4 = rays[2 * rid], d4 = rays[2 * rid + 1];
                    v3 o(o4.x, o4.y, o4.z), d(d4.x, d4.y, d4.z);
                    float t = d4.w;
                    light = -1;
                    bool done = false;
                    if (lights)
                    {
                        if (kAny)
                            done = lights_any(S, o, d, t);
                        else
                            t = lights_closest(S, o, d, t, &light);
                    }
                    trav_init(s, S, o, d, t);
                    if (done)
                    {
                        occluded[rid] = 1;
                        rid = -1;
                    }
                }
                else
                    rid = -2;
            }
        }
        if (__all_sync(kFullMask, rid == -2)) break;
        if (rid >= 0 && trav_run<kAny>(s, S, 32))
        {
            if (kAny)
                occluded[rid] = s.hitPrim >= 0 ? 1 : 0;
            else
                hits[rid] = make_int4(__float_as_int(s.t), s.hitInst, s.hitPrim, s.hitPrim >= 0 ? -1 : light);
            if (s.err) atomicOr(status, s.err);
            rid = -1;
        }
    }
}

// Wide-tree form: each lane traces its ray to completion; warps take rays 32 at a time from a
// global counter (in `perm` order), so a warp that finished early takes more work. (Refilling
// single lanes as their rays end, with the traversal state kept in registers, measured 35 %
// slower: the binned rays of a warp stop sharing nodes and the refill logic spills.)
template <bool kAny>
__global__ void __launch_bounds__(128) trace_fetch_wide_kernel(DevScene S, const float4* rays, const int* perm,
                                                               long long n, int4* hits, uint8_t* occluded, int lights,
                                                               unsigned long long* next, uint32_t* status)
{
    const int lane = threadIdx.x & 31;
    while (true)
    {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(next, 32ull);
        base = __shfl_sync(kFullMask, base, 0);
        if (base >= (unsigned long long)n) break;
        const unsigned long long my = base + lane;
        if (my < (unsigned long long)n)
        {
            const long long rid = perm ? (long long)perm[my] : (long long)my;
            const float4 o4 = rays[2 * rid], d4 = rays[2 * rid + 1];
            const v3 o(o4.x, o4.y, o4.z), d(d4.x, d4.y, d4.z);
            Hit h;
            uint32_t err;
            if (kAny)
            {
                bool occ;
                err = any_hit<false>(S, o, d, d4.w, lights != 0, &occ, &h, nullptr);
                occluded[rid] = occ ? 1 : 0;
            }
            else
            {
                err = closest_hit<false>(S, o, d, d4.w, lights != 0, &h, nullptr);
                hits[rid] = make_int4(__float_as_int(h.t), h.inst, h.prim, h.light);
            }
            if (err) atomicOr(status, err);
        }
    }
}

int launch_trace_binned(const DevScene& S, const float4* rays, long long n, void* out, bool any, int lights,
                        const float lo[3], const float hi[3], bool binning, uint32_t* keys, uint32_t* hist, int* perm,
                        unsigned long long* next, uint32_t* status, cudaStream_t st, cudaEvent_t evStart,
                        cudaEvent_t evStop)
{
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int* order = nullptr;
    if (binning)
    {
        float3 flo = make_float3(lo[0], lo[1], lo[2]);
        auto inv = [](float a, float b) { return b > a ? (float)kCells / (b - a) : 0.0f; };
        float3 finv = make_float3(inv(lo[0], hi[0]), inv(lo[1], hi[1]), inv(lo[2], hi[2]));
        cudaMemsetAsync(hist, 0, sizeof(uint32_t) * kBins, st);
        int g = sms * 8;
        ray_keys_kernel<<<g, 256, 0, st>>>(rays, n, flo, finv, keys, hist);
        bins_scan_kernel<<<kScanBlocks, kScanBlock, 0, st>>>(hist);
        bins_scan_totals_kernel<<<1, kScanBlock, 0, st>>>(hist);
        bins_scan_add_kernel<<<kScanBlocks, kScanBlock, 0, st>>>(hist);
        ray_scatter_kernel<<<g, 256, 0, st>>>(keys, n, hist, perm);
        order = perm;
    }
    cudaMemsetAsync(next, 0, sizeof(unsigned long long), st);
    int per_sm = 0;
    if (S.wnodes && S.wideOn)
    {
        if (any)
        {
            per_sm = occupancy_blocks_per_sm((const void*)trace_fetch_wide_kernel<true>, 128);
            if (evStart) cudaEventRecord(evStart, st);
            trace_fetch_wide_kernel<true><<<sms * (per_sm > 0 ? per_sm : 1), 128, 0, st>>>(
                S, rays, order, n, nullptr, (uint8_t*)out, lights, next, status);
        }
        else
        {
            per_sm = occupancy_blocks_per_sm((const void*)trace_fetch_wide_kernel<false>, 128);
            if (evStart) cudaEventRecord(evStart, st);
            trace_fetch_wide_kernel<false><<<sms * (per_sm > 0 ? per_sm : 1), 128, 0, st>>>(
                S, rays, order, n, (int4*)out, nullptr, lights, next, status);
        }
        if (evStop) cudaEventRecord(evStop, st);
        return (int)cudaGetLastError();
    }
    if (evStart) cudaEventRecord(evStart, st);
    if (any)
    {
        per_sm = occupancy_blocks_per_sm((const void*)trace_persistent_kernel<true>, 128);
        trace_persistent_kernel<true><<<sms * (per_sm > 0 ? per_sm : 1), 128, 0, st>>>(
            S, rays, order, n, nullptr, (uint8_t*)out, lights, next, status);
    }
    else
    {
        per_sm = occupancy_blocks_per_sm((const void*)trace_persistent_kernel<false>, 128);
        trace_persistent_kernel<false><<<sms * (per_sm > 0 ? per_sm : 1), 128, 0, st>>>(
            S, rays, order, n, (int4*)out, nullptr, lights, next, status);
    }
    if (evStop) cudaEventRecord(evStop, st);
    return (int)cudaGetLastError();
}

int trace_bins() { return kBins + kScanBlocks; }   // counters + scan partial sums
}
