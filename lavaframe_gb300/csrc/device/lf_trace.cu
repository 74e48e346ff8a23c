// Batched ray queries (ClosestHit / AnyHit as a service): ray binning and a persistent
// traversal kernel.
//
// Random rays give each lane of a warp its own path through the BVH: few lanes share an
// instruction and almost every node comes from DRAM. Two measures, neither of which changes
// any per-ray result:
//  - binning: rays are counting-sorted by a key made of the Morton code of their origin
//    cell (32^3 cells over the scene box) and their direction octant, so neighbouring lanes
//    start in the same region heading the same way and share nodes in L1/L2;
//  - persistent warps with dynamic fetch: each warp keeps its 32 lanes busy by giving a new
//    ray to every lane whose ray finished (one atomic per warp refill), instead of waiting
//    for the slowest ray of a fixed batch.
#include "lf_kernels.h"

namespace lfd
{
namespace
{
constexpr unsigned kFullMask = 0xffffffffu;
constexpr int kBinBits = 18;   // 15 bits of origin Morton code + 3 bits of octant
constexpr int kBins = 1 << kBinBits;

__device__ __forceinline__ uint32_t spread3(uint32_t x)   // 5 bits -> every third bit
{
    x &= 31u;
    x = (x | (x << 8)) & 0x0000F00Fu;
    x = (x | (x << 4)) & 0x000C30C3u;
    x = (x | (x << 2)) & 0x00249249u;
    return x;
}

__device__ __forceinline__ uint32_t cell(float v, float lo, float inv)
{
    float q = (v - lo) * inv;
    q = q < 0.f ? 0.f : (q > 31.f ? 31.f : q);
    return (uint32_t)q;
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

// Exclusive scan of kBins counters by one block of 1024 threads.
__global__ void bins_scan_kernel(uint32_t* hist)
{
    __shared__ uint32_t part[1024];
    const int per = kBins / 1024;
    const int t = threadIdx.x;
    uint32_t sum = 0;
    for (int i = 0; i < per; ++i) sum += hist[t * per + i];
    part[t] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1)
    {
        uint32_t v = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = part[t] - sum;
    for (int i = 0; i < per; ++i)
    {
        uint32_t c = hist[t * per + i];
        hist[t * per + i] = run;
        run += c;
    }
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
                        unsigned long long* next, uint32_t* status, cudaStream_t st)
{
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int* order = nullptr;
    if (binning)
    {
        float3 flo = make_float3(lo[0], lo[1], lo[2]);
        auto inv = [](float a, float b) { return b > a ? 32.0f / (b - a) : 0.0f; };
        float3 finv = make_float3(inv(lo[0], hi[0]), inv(lo[1], hi[1]), inv(lo[2], hi[2]));
        cudaMemsetAsync(hist, 0, sizeof(uint32_t) * kBins, st);
        int g = sms * 8;
        ray_keys_kernel<<<g, 256, 0, st>>>(rays, n, flo, finv, keys, hist);
        bins_scan_kernel<<<1, 1024, 0, st>>>(hist);
        ray_scatter_kernel<<<g, 256, 0, st>>>(keys, n, hist, perm);
        order = perm;
    }
    cudaMemsetAsync(next, 0, sizeof(unsigned long long), st);
    int per_sm = 0;
    if (S.wnodes && S.wideOn)
    {
        if (any)
        {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trace_fetch_wide_kernel<true>, 128, 0);
            trace_fetch_wide_kernel<true><<<sms * (per_sm > 0 ? per_sm : 1), 128, 0, st>>>(
                S, rays, order, n, nullptr, (uint8_t*)out, lights, next, status);
        }
        else
        {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trace_fetch_wide_kernel<false>, 128, 0);
            trace_fetch_wide_kernel<false><<<sms * (per_sm > 0 ? per_sm : 1), 128, 0, st>>>(
                S, rays, order, n, (int4*)out, nullptr, lights, next, status);
        }
        return (int)cudaGetLastError();
    }
    if (any)
    {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trace_persistent_kernel<true>, 128, 0);
        trace_persistent_kernel<true><<<sms * (per_sm > 0 ? per_sm : 1), 128, 0, st>>>(
            S, rays, order, n, nullptr, (uint8_t*)out, lights, next, status);
    }
    else
    {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trace_persistent_kernel<false>, 128, 0);
        trace_persistent_kernel<false><<<sms * (per_sm > 0 ? per_sm : 1), 128, 0, st>>>(
            S, rays, order, n, (int4*)out, nullptr, lights, next, status);
    }
    return (int)cudaGetLastError();
}

int trace_bins() { return kBins; }
}
