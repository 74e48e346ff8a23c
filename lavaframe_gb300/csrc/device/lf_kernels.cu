// Wavefront path-tracing kernels and batched ray queries.
//
// Pipeline per batch of samples (one path per pixel and sample):
//   generate  camera ray + RNG per path, all paths queued           (renderer.glsl:25-62)
//   extend    closest hit for every queued path                     (closest_hit.glsl)
//   shade     surface/miss/emitter logic, next-event candidates, BSDF sample, Russian
//             roulette; survivors compacted into the next queue     (pathtrace.glsl:208-294)
//   shadow    occlusion of the next-event rays, adds DirectLight*T (pathtrace.glsl:126-204)
//   accumulate per-pixel sum over the batch's samples in sample order (renderer.glsl:64-68)
// Path state lives in SoA arrays in HBM; queues are compacted with one atomic per warp
// (ballot + popc). Every kernel runs a warp-uniform grid-stride loop over a device-side
// count, so the bounce loop needs no host round trip and can be captured in a graph.
#include <mutex>
#include <vector>

#include "lf_pathops.cuh"

namespace lfd
{
using namespace pathops;


// ------------------------------------------------------------------ generate
// Slot s * tilePix + lp starts sample s of tile pixel pixel_of(lp) (8 x 4 blocks), so a
// warp's camera rays cover a compact patch; info.x holds the pixel for the accumulation.
__global__ void generate_kernel(ShadeScene S, Params P, PathSoA ps, int firstSample, int nSamples, int* queue,
                                int* qcount)
{
    const int tilePix = P.tileW * P.tileH;
    const long long n = (long long)nSamples * tilePix;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long warpBase = ((long long)blockIdx.x * blockDim.x + threadIdx.x) & ~31ll;
    const int lane = threadIdx.x & 31;
    for (long long base = warpBase; base < n; base += stride)
    {
        long long i = base + lane;
        bool push = false;
        int slot = (int)i;
        if (i < n)
        {
            int s = (int)(i / tilePix);
            int lp = (int)(i - (long long)s * tilePix);
            int lx, ly;
            pixel_of(lp, P.tileW, P.tileH, lx, ly);   // the same pixel for every sample of lp
            int gx = P.tileX * P.tileW + lx, gy = P.tileY * P.tileH + ly;
            bool inside = gx < P.width && gy < P.height;
            ps.L[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
            ps.info[slot] = make_int4(inside ? gy * P.width + gx : -1, 0, 0, 0);
            if (inside)
            {
                gen_path(P, P.tileX, P.tileY, P.tileOrdinal, firstSample + s, lx, ly, ps, slot);
                push = true;
            }
        }
        warp_push(push, slot, queue, qcount, (int)n, nullptr);
    }
}

// ------------------------------------------------------------------ extend
// Warps take queue entries 32 at a time from `fetch`; 72 registers (7 blocks of 128 per SM).
__global__ void __maxnreg__(72) extend_kernel(ShadeScene S, Params P, PathSoA ps, const int* queue, const int* qcount,
                                              unsigned long long* fetch, uint32_t* status, unsigned long long* ctr)
{
    const int n = *qcount;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ctr[1], (unsigned long long)n);
    const bool lights = P.useLights != 0;
    const int lane = threadIdx.x & 31;
    while (true)
    {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(fetch, 32ull);
        base = __shfl_sync(kFull, base, 0);
        if (base >= (unsigned long long)n) break;
        const int i = (int)base + lane;
        if (i >= n) continue;
        int p = queue[i];
        float4 o4 = ps.o[p], d4 = ps.d[p];
        Hit h;
        uint32_t err = closest_hit<false>(S.trav, f3(o4), f3(d4), kInfinity, lights, &h, nullptr);
        ps.hit[p] = make_float4(h.t, __int_as_float(h.inst), __int_as_float(h.prim), __int_as_float(h.light));
        set_error(status, err);
    }
}

// ------------------------------------------------------------------ shade
// 8 blocks of 128 threads per SM: caps registers at 64 (some spills; 9 % faster on the 1M-
// triangle render than 128 registers without spills).
template <bool kLights>
__global__ void __launch_bounds__(128, 8) shade_kernel(ShadeScene S, Params P, PathSoA ps, const int* qin,
                                                        const int* qinCount, int* qout, int* qoutCount, ShadowRec* sq,
                                                        int* sqCount, int cap, uint32_t* status,
                                                        unsigned long long* ctr)
{
    const int n = *qinCount;
    const int stride = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    const int warpBase = (blockIdx.x * blockDim.x + threadIdx.x) & ~31;
    for (int base = warpBase; base < n; base += stride)
    {
        int i = base + lane;
        bool pushExt = false, pushShadow = false;
        int p = -1;
        ShadowRec rec;
        if (i < n)
        {
            p = qin[i];
            shade_path<kLights>(S, P, ps, p, ctr, pushExt, pushShadow, rec);
        }
        warp_push(pushExt, p, qout, qoutCount, cap, status);
        warp_push(pushShadow, rec, sq, sqCount, cap, status);
    }
}

// ------------------------------------------------------------------ shadow
__global__ void __maxnreg__(72) shadow_kernel(ShadeScene S, Params P, PathSoA ps, const ShadowRec* sq,
                                              const int* sqCount, unsigned long long* fetch, uint32_t* status,
                                              unsigned long long* ctr)
{
    const int n = *sqCount;
    unsigned long long rays = 0;
    const int lane = threadIdx.x & 31;
    while (true)
    {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(fetch, 32ull);
        base = __shfl_sync(kFull, base, 0);
        if (base >= (unsigned long long)n) break;
        const int i = (int)base + lane;
        if (i < n) set_error(status, shadow_path(S, P, ps, sq + i, rays));
    }
    warp_count_add(&ctr[2], rays);
}

// ------------------------------------------------------------------ accumulate
__global__ void accumulate_kernel(Params P, PathSoA ps, int nSamples, float4* accum, double* accum64)
{
    const int tilePix = P.tileW * P.tileH;
    for (int lp = blockIdx.x * blockDim.x + threadIdx.x; lp < tilePix; lp += gridDim.x * blockDim.x)
    {
        int gpix = ps.info[lp].x;
        if (gpix < 0) continue;
        float4 a = accum[gpix];
        double ax = 0, ay = 0, az = 0;
        if (accum64)
        {
            ax = accum64[gpix * 3 + 0];
            ay = accum64[gpix * 3 + 1];
            az = accum64[gpix * 3 + 2];
        }
        for (int s = 0; s < nSamples; ++s)
        {
            float4 l = ps.L[(size_t)s * tilePix + lp];
            a.x = a.x + l.x;
            a.y = a.y + l.y;
            a.z = a.z + l.z;
            if (accum64)
            {
                ax += (double)l.x;
                ay += (double)l.y;
                az += (double)l.z;
            }
        }
        accum[gpix] = a;
        if (accum64)
        {
            accum64[gpix * 3 + 0] = ax;
            accum64[gpix * 3 + 1] = ay;
            accum64[gpix * 3 + 2] = az;
        }
    }
}

// ------------------------------------------------------------------ ray queries
template <bool kStats>
__global__ void trace_closest_kernel(DevScene S, const float4* rays, long long n, int4* hits, int lights,
                                     uint32_t* status, unsigned long long* stats)
{
    TraceStats st{0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    {
        float4 o4 = rays[2 * i], d4 = rays[2 * i + 1];
        Hit h;
        uint32_t err = closest_hit<kStats>(S, f3(o4), f3(d4), d4.w, lights != 0, &h, &st);
        hits[i] = make_int4(__float_as_int(h.t), h.inst, h.prim, h.light);
        set_error(status, err);
    }
    if (kStats)
    {
        atomicAdd(&stats[0], st.nodes);
        atomicAdd(&stats[1], st.tris);
        atomicAdd(&stats[2], st.leaves);
    }
}

template <bool kStats>
__global__ void trace_any_kernel(DevScene S, const float4* rays, long long n, uint8_t* occluded, int lights,
                                 uint32_t* status, unsigned long long* stats)
{
    TraceStats st{0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    {
        float4 o4 = rays[2 * i], d4 = rays[2 * i + 1];
        Hit h;
        bool occ;
        uint32_t err = any_hit<kStats>(S, f3(o4), f3(d4), d4.w, lights != 0, &occ, &h, &st);
        occluded[i] = occ ? 1 : 0;
        set_error(status, err);
    }
    if (kStats)
    {
        atomicAdd(&stats[0], st.nodes);
        atomicAdd(&stats[1], st.tris);
        atomicAdd(&stats[2], st.leaves);
    }
}

// ------------------------------------------------------------------ guided bounces
// Query record (position, outgoing direction, shading normal) of every queued path that hit a
// triangle; other entries get a zero record (their mixture is computed and not used).
// pixelShare > 0 (the first bounce of a batch of several samples): one query per pixel, from the
// pixel's sample-0 path (slot p < pixelShare), stored at the pixel's index; the other queued
// paths write none.
__global__ void guide_query_kernel(ShadeScene S, PathSoA ps, const int* queue, const int* qcount, float* queries,
                                   int pixelShare)
{
    const int n = *qcount;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const int p = queue[i];
        if (pixelShare > 0 && p >= pixelShare) continue;
        const float4 h = ps.hit[p];
        float* q = queries + (size_t)(pixelShare > 0 ? p : i) * guide::kSampleFloats;
        float v[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 1.f};
        const int prim = __float_as_int(h.z), light = __float_as_int(h.w);
        if (h.x != kInfinity && light < 0 && prim >= 0)
        {
            const float4 o4 = ps.o[p], d4 = ps.d[p];
            const SurfaceGeom g = surface_geom(S, f3(o4), f3(d4), h.x, __float_as_int(h.y), prim);
            const float vv[9] = {g.fhp.x, g.fhp.y, g.fhp.z, -d4.x, -d4.y, -d4.z, g.nrm.x, g.nrm.y, g.nrm.z};
            for (int k = 0; k < 9; ++k) v[k] = vv[k];
        }
        for (int k = 0; k < 9; ++k) q[k] = v[k];
    }
}

// pixelShare > 0: the mixtures are per pixel (guide_query_kernel's pixelShare), path p uses its
// pixel's, p % pixelShare.
__global__ void __launch_bounds__(128, 4) shade_guided_kernel(ShadeScene S, Params P, PathSoA ps, const int* qin,
                                                               const int* qinCount, int* qout, int* qoutCount,
                                                               ShadowRec* sq, int* sqCount, int cap, uint32_t* status,
                                                               unsigned long long* ctr, GuideCtx gc, int pixelShare)
{
    const int n = *qinCount;
    const int stride = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    const int warpBase = (blockIdx.x * blockDim.x + threadIdx.x) & ~31;
    for (int base = warpBase; base < n; base += stride)
    {
        int i = base + lane;
        bool pushExt = false, pushShadow = false;
        int p = -1;
        ShadowRec rec;
        if (i < n)
        {
            p = qin[i];
            shade_path_t<true>(S, P, ps, p, ctr, pushExt, pushShadow, rec, gc, pixelShare > 0 ? p % pixelShare : i);
        }
        warp_push(pushExt, p, qout, qoutCount, cap, status);
        warp_push(pushShadow, rec, sq, sqCount, cap, status);
    }
}

// Training samples of the batch: for every recorded vertex k of a path (all but the path's
// last vertex), the radiance its sampled direction carried is (L_final - L_start(k+1)) /
// throughput after k; the sample weight is its luminance over the direction's pdf.
__global__ void guide_collect_kernel(PathSoA ps, GuideBuffers g, long long n)
{
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = ((long long)blockIdx.x * blockDim.x + threadIdx.x) & ~31ll; base < n; base += stride)
    {
        const long long p = base + lane;
        int depth = 0;
        float4 Lf = make_float4(0.f, 0.f, 0.f, 0.f);
        if (p < n && ps.info[p].x >= 0)
        {
            depth = ps.info[p].y;
            Lf = ps.L[p];
        }
        const int maxK = __reduce_max_sync(kFull, (unsigned)(depth > 1 ? depth - 1 : 0));
        for (int k = 0; k < maxK; ++k)
        {
            bool take = false;
            float smp[13];
            if (k < depth - 1)
            {
                auto r = [&](int f) { return *guide_rec(g.rec, n, (int)p, k, f); };
                const float pdf = r(12);
                if (r(19) == 2.f && pdf > 0.f)
                {
                    const float tx = r(13), ty = r(14), tz = r(15);
                    const float lx = tx > 0.f ? (Lf.x - r(16)) / tx : 0.f;
                    const float ly = ty > 0.f ? (Lf.y - r(17)) / ty : 0.f;
                    const float lz = tz > 0.f ? (Lf.z - r(18)) / tz : 0.f;
                    const float lum = 0.2126f * lx + 0.7152f * ly + 0.0722f * lz;
                    const float w = fminf(lum / pdf, g.weightClamp);
                    if (w > 0.f && w == w)
                    {
#pragma unroll
                        for (int c = 0; c < 12; ++c) smp[c] = r(c);
                        smp[12] = w;
                        take = true;
                    }
                }
            }
            const unsigned m = __ballot_sync(kFull, take);
            if (!m) continue;
            const int leader = __ffs(m) - 1;
            int pos0 = 0;
            if (lane == leader) pos0 = atomicAdd(g.trainCount, __popc(m));
            pos0 = __shfl_sync(kFull, pos0, leader);
            if (take)
            {
                const int pos = pos0 + __popc(m & ((1u << lane) - 1u));
                if (pos < g.trainCap)
                {
                    float* dst = g.train + (size_t)pos * guide::kSampleFloats;
                    for (int c = 0; c < 13; ++c) dst[c] = smp[c];
                    dst[13] = dst[14] = dst[15] = 0.f;
                }
            }
        }
    }
}

// ------------------------------------------------------------------ launchers
namespace
{
int g_num_sms = 0;

int grid_for(const void* kernel, int block, long long work)
{
    if (g_num_sms == 0)
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    const int per_sm = occupancy_blocks_per_sm(kernel, block);
    long long full = (long long)g_num_sms * per_sm;
    long long need = (work + block - 1) / block;
    if (need < 1) need = 1;
    return (int)(need < full ? need : full);
}
}

int occupancy_blocks_per_sm(const void* kernel, int block, size_t dynamicSmem)
{
    struct Entry
    {
        const void* kernel;
        int block, perSm, device;
        size_t smem;
    };
    static std::mutex mu;
    static std::vector<Entry> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> lk(mu);
        for (const Entry& e : cache)
            if (e.kernel == kernel && e.block == block && e.device == dev && e.smem == dynamicSmem) return e.perSm;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, dynamicSmem);
    if (per_sm <= 0) per_sm = 1;
    std::lock_guard<std::mutex> lk(mu);
    cache.push_back({kernel, block, per_sm, dev, dynamicSmem});
    return per_sm;
}

int launch_generate(const ShadeScene& S, const Params& P, const PathSoA& ps, int firstSample, int nSamples,
                    int* queue, int* qcount, cudaStream_t st)
{
    const int B = 256;
    long long work = (long long)nSamples * P.tileW * P.tileH;
    int g = grid_for((const void*)generate_kernel, B, work);
    generate_kernel<<<g, B, 0, st>>>(S, P, ps, firstSample, nSamples, queue, qcount);
    return (int)cudaGetLastError();
}

int launch_bounce(const ShadeScene& S, const Params& P, const PathSoA& ps, const BounceBuffers& b, int bounce,
                  long long cap, cudaStream_t st)
{
    int* qin = b.queue[bounce & 1];
    int* qout = b.queue[(bounce + 1) & 1];
    int* cin = b.count + (bounce & 1);
    int* cout = b.count + ((bounce + 1) & 1);
    cudaMemsetAsync(cout, 0, sizeof(int), st);
    cudaMemsetAsync(b.shadowCount, 0, sizeof(int), st);
    const int BE = 128, BS = 128, BW = 128;
    cudaMemsetAsync(b.fetch, 0, 2 * sizeof(unsigned long long), st);
    int ge = grid_for((const void*)extend_kernel, BE, cap);
    extend_kernel<<<ge, BE, 0, st>>>(S, P, ps, qin, cin, b.fetch, b.status, b.ctr);
    if (P.useLights)
    {
        int gs = grid_for((const void*)shade_kernel<true>, BS, cap);
        shade_kernel<true><<<gs, BS, 0, st>>>(S, P, ps, qin, cin, qout, cout, b.shadow, b.shadowCount, (int)cap, b.status,
                                              b.ctr);
    }
    else
    {
        int gs = grid_for((const void*)shade_kernel<false>, BS, cap);
        shade_kernel<false><<<gs, BS, 0, st>>>(S, P, ps, qin, cin, qout, cout, b.shadow, b.shadowCount, (int)cap,
                                               b.status, b.ctr);
    }
    int gw = grid_for((const void*)shadow_kernel, BW, cap);
    shadow_kernel<<<gw, BW, 0, st>>>(S, P, ps, b.shadow, b.shadowCount, b.fetch + 1, b.status, b.ctr);
    return (int)cudaGetLastError();
}

int launch_bounce_guided(const ShadeScene& S, const Params& P, const PathSoA& ps, const BounceBuffers& b,
                         const GuideBuffers& g, int bounce, long long cap, cudaStream_t st)
{
    int* qin = b.queue[bounce & 1];
    int* qout = b.queue[(bounce + 1) & 1];
    int* cin = b.count + (bounce & 1);
    int* cout = b.count + ((bounce + 1) & 1);
    cudaMemsetAsync(cout, 0, sizeof(int), st);
    cudaMemsetAsync(b.shadowCount, 0, sizeof(int), st);
    const int B = 128;
    cudaMemsetAsync(b.fetch, 0, 2 * sizeof(unsigned long long), st);
    extend_kernel<<<grid_for((const void*)extend_kernel, B, cap), B, 0, st>>>(S, P, ps, qin, cin, b.fetch, b.status,
                                                                              b.ctr);
    // First bounce of a batch of several samples: the samples of a pixel hit its footprint
    // from the same camera, so they share one mixture, inferred from the pixel's sample-0 path
    // (a proposal that does not depend on the other samples' own draws keeps them unbiased).
    const long long tilePix = (long long)P.tileW * P.tileH;
    const int share = bounce == 0 && cap > tilePix ? (int)tilePix : 0;
    guide_query_kernel<<<grid_for((const void*)guide_query_kernel, B, cap), B, 0, st>>>(S, ps, qin, cin, g.queries,
                                                                                      share);
    const int* nq = share ? nullptr : cin;
    const int qcap = share ? share : (int)cap;
    int e = g.tensorPath ? guide::launch_infer_tc(g.net, g.queries, nq, qcap, g.mix, b.status, st)
                         : guide::launch_infer(g.net, g.queries, nq, qcap, g.mix, st);
    if (e) return e;
    GuideCtx gc{g.mix, g.rec, g.alpha, g.maxDepth, cap};
    shade_guided_kernel<<<grid_for((const void*)shade_guided_kernel, B, cap), B, 0, st>>>(
        S, P, ps, qin, cin, qout, cout, b.shadow, b.shadowCount, (int)cap, b.status, b.ctr, gc, share);
    shadow_kernel<<<grid_for((const void*)shadow_kernel, B, cap), B, 0, st>>>(S, P, ps, b.shadow, b.shadowCount,
                                                                             b.fetch + 1, b.status, b.ctr);
    return (int)cudaGetLastError();
}

int launch_guide_collect(const PathSoA& ps, const GuideBuffers& g, long long n, cudaStream_t st)
{
    guide_collect_kernel<<<grid_for((const void*)guide_collect_kernel, 256, n), 256, 0, st>>>(ps, g, n);
    return (int)cudaGetLastError();
}

int launch_accumulate(const Params& P, const PathSoA& ps, int nSamples, float4* accum, double* accum64,
                      cudaStream_t st)
{
    const int B = 256;
    int g = grid_for((const void*)accumulate_kernel, B, (long long)P.tileW * P.tileH);
    accumulate_kernel<<<g, B, 0, st>>>(P, ps, nSamples, accum, accum64);
    return (int)cudaGetLastError();
}

int launch_trace_closest(const DevScene& S, const float4* rays, long long n, int4* hits, int lights, bool stats,
                         uint32_t* status, unsigned long long* stat3, cudaStream_t st)
{
    const int B = 128;
    if (stats)
    {
        int g = grid_for((const void*)trace_closest_kernel<true>, B, n);
        trace_closest_kernel<true><<<g, B, 0, st>>>(S, rays, n, hits, lights, status, stat3);
    }
    else
    {
        int g = grid_for((const void*)trace_closest_kernel<false>, B, n);
        trace_closest_kernel<false><<<g, B, 0, st>>>(S, rays, n, hits, lights, status, stat3);
    }
    return (int)cudaGetLastError();
}

int launch_trace_any(const DevScene& S, const float4* rays, long long n, uint8_t* occ, int lights, bool stats,
                     uint32_t* status, unsigned long long* stat3, cudaStream_t st)
{
    const int B = 128;
    if (stats)
    {
        int g = grid_for((const void*)trace_any_kernel<true>, B, n);
        trace_any_kernel<true><<<g, B, 0, st>>>(S, rays, n, occ, lights, status, stat3);
    }
    else
    {
        int g = grid_for((const void*)trace_any_kernel<false>, B, n);
        trace_any_kernel<false><<<g, B, 0, st>>>(S, rays, n, occ, lights, status, stat3);
    }
    return (int)cudaGetLastError();
}
}
