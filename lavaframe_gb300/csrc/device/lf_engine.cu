// Kernels of the persistent multi-job wavefront engine (tables and step order in lf_engine.h).
// The per-path work is the same code as the per-batch frame kernels (lf_pathops.cuh); only
// the bookkeeping differs: paths find their job through info.w, finished paths hand their
// slot to a new path, and pass completion is counted on the device.
#include "lf_engine.h"
#include "lf_pathops.cuh"

namespace lfd
{
using namespace pathops;

namespace
{
__device__ __forceinline__ int job_of(int w) { return (int)((unsigned)w >> kPassRingBits); }
__device__ __forceinline__ int ring_of(int w) { return w & (kPassRing - 1); }

// Pass completion counts of a block: a small shared table keyed by ring entry, added into
// passDone once per block at its end (an entry that finds the table full goes straight to the
// global counter).
struct DoneTable
{
    int key[8];
    unsigned cnt[8];
};

__device__ __forceinline__ void done_table_add(DoneTable& t, int ring, unsigned c, unsigned long long* passDone)
{
    if (ring < 0 || c == 0) return;
    for (int k = 0; k < 8; ++k)
    {
        const int e = (ring + k) & 7;
        const int old = atomicCAS(&t.key[e], -1, ring);
        if (old == -1 || old == ring)
        {
            atomicAdd(&t.cnt[e], c);
            return;
        }
    }
    atomicAdd(&passDone[ring], (unsigned long long)c);
}

// Per-block completion bookkeeping of the kernels that end paths (finish, shade, shadow,
// drain): completions summed per thread while the ring entry repeats, per block in a shared
// table, and into the global counters once per block at its end.
struct BlockDone
{
    DoneTable table;
    unsigned written;
};

__device__ __forceinline__ void block_done_begin(BlockDone& bd)
{
    if (threadIdx.x < 8)
    {
        bd.table.key[threadIdx.x] = -1;
        bd.table.cnt[threadIdx.x] = 0;
    }
    if (threadIdx.x == 0) bd.written = 0;
    __syncthreads();
}

struct ThreadDone
{
    int run = -1;
    unsigned runCount = 0, written = 0;
};

// Writes out the final radiance L of the path in `slot` into its pass's buffer, frees the slot
// and counts the completion.
__device__ __forceinline__ void end_path(const EngineBuffers& b, int slot, const int4& inf, const float4& L,
                                         ThreadDone& td, BlockDone& bd)
{
    const int ring = ring_of(inf.w);
    b.passes[ring].radiance[inf.x] = L;
    reinterpret_cast<int*>(b.ps.info)[4 * slot + 3] = -1;
    if (ring != td.run)
    {
        done_table_add(bd.table, td.run, td.runCount, b.passDone);
        td.run = ring;
        td.runCount = 0;
    }
    ++td.runCount;
    ++td.written;
}

// Every thread of the block must call, once, after its last end_path.
__device__ __forceinline__ void block_done_end(const EngineBuffers& b, const ThreadDone& td, BlockDone& bd)
{
    done_table_add(bd.table, td.run, td.runCount, b.passDone);
    const unsigned w = __reduce_add_sync(kFull, td.written);
    if ((threadIdx.x & 31) == 0 && w) atomicAdd(&bd.written, w);
    __syncthreads();
    if (threadIdx.x < 8 && bd.table.key[threadIdx.x] >= 0 && bd.table.cnt[threadIdx.x])
        atomicAdd(&b.passDone[bd.table.key[threadIdx.x]], (unsigned long long)bd.table.cnt[threadIdx.x]);
    if (threadIdx.x == 0 && bd.written)
    {
        atomicSub(&b.ctl->active, (int)bd.written);
        atomicAdd(&b.ctl->freeCount, (int)bd.written);
    }
}

// Largest pass g in [lo, hi) with pathBase <= id (passes are in increasing pathBase order).
__device__ __forceinline__ unsigned long long find_pass(const EnginePass* passes, unsigned long long id,
                                                        unsigned long long lo, unsigned long long hi)
{
    while (hi - lo > 1)
    {
        const unsigned long long mid = lo + ((hi - lo) >> 1);
        if (passes[mid & (kPassRing - 1)].pathBase <= id) lo = mid;
        else hi = mid;
    }
    return lo;
}
}

// ------------------------------------------------------------------ init / append / reset
__global__ void engine_init_kernel(EngineBuffers b)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < b.cap; i += gridDim.x * blockDim.x)
    {
        b.ps.info[i] = make_int4(0, 0, 0, -1);   // info.w = -1: the slot is free
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        b.ctl->freeCount = b.cap;
        b.ctl->taken = 0;
        b.ctl->doneCount[0] = 0;
        b.ctl->doneCount[1] = 0;
        b.ctl->active = 0;
        b.ctl->count[0] = 0;
        b.ctl->count[1] = 0;
        b.ctl->shadowCount = 0;
    }
}

__global__ void engine_append_kernel(EngineBuffers b, unsigned long long total, unsigned long long numPasses)
{
    EngineCtl* c = b.ctl;
    const unsigned long long next = c->next;
    c->total = total;
    c->numPasses = numPasses;
    unsigned long long lo = c->passLo;
    while (lo + 1 < numPasses)
    {
        const EnginePass& q = b.passes[lo & (kPassRing - 1)];
        if (q.pathBase + q.numPaths > next) break;
        ++lo;
    }
    c->passLo = lo;
}

// After finish and refill: count the refilled slots as taken and their ids as issued, and
// clear the lists and counters the rest of the step fills.
__global__ void engine_reset_kernel(EngineCtl* c, int parity)
{
    c->freeCount -= c->taken;
    c->next += (unsigned long long)c->taken;
    c->active += c->taken;
    c->taken = 0;
    c->doneCount[parity] = 0;
    c->shadowCount = 0;
    c->count[parity ^ 1] = 0;
    c->extendNext = 0;
    c->shadeNext = 0;
    c->shadowNext = 0;
    c->refillNext = 0;
    c->hitCount = 0;
    c->missCount = 0;
    for (int k = 0; k < 4; ++k) c->bucketCount[k] = 0;
}

// ------------------------------------------------------------------ finish / refill
constexpr int kFinishUnroll = 4;   // done entries a thread has in flight
constexpr int kRefillBlock = 256;  // refill block size (8 warps)
constexpr int kRefillGroups = 4;   // groups of kRefillBlock slots a refill block takes per scan step

// Writes out the radiance of the paths on the done list (paths of depth-0 jobs; the step
// kernels end every other path where it ends), counting pass completions, and frees their
// slots. A thread loads four entries' state before it writes any.
__global__ void __launch_bounds__(256) engine_finish_kernel(EngineBuffers b, int parity)
{
    __shared__ BlockDone bd;
    block_done_begin(bd);
    ThreadDone td;
    const int n = b.ctl->doneCount[parity];
    const int* done = b.done[parity];
    const int stride = gridDim.x * blockDim.x;
    for (int i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += kFinishUnroll * stride)
    {
        int slot[kFinishUnroll];
        int4 inf[kFinishUnroll];
        float4 L[kFinishUnroll];
#pragma unroll
        for (int u = 0; u < kFinishUnroll; ++u)
        {
            const int i = i0 + u * stride;
            slot[u] = i < n ? done[i] : -1;
        }
#pragma unroll
        for (int u = 0; u < kFinishUnroll; ++u)
            if (slot[u] >= 0)
            {
                inf[u] = b.ps.info[slot[u]];
                L[u] = b.ps.L[slot[u]];
            }
#pragma unroll
        for (int u = 0; u < kFinishUnroll; ++u)
            if (slot[u] >= 0) end_path(b, slot[u], inf[u], L[u], td, bd);
    }
    block_done_end(b, td, bd);
}

// Exclusive scan of one int per lane; returns the warp total. All 32 lanes must call.
__device__ __forceinline__ int warp_exclusive_scan(int& v)
{
    const int lane = threadIdx.x & 31;
    int incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1)
    {
        const int u = __shfl_up_sync(kFull, incl, d);
        if (lane >= d) incl += u;
    }
    const int total = __shfl_sync(kFull, incl, 31);
    v = incl - v;
    return total;
}

// Starts min(free slots, unissued ids) new paths in free slots taken in slot order: the pool is
// scanned in steps of kRefillGroups x kRefillBlock slots per block, a step's free slots get
// consecutive ids (next + k for the k-th slot handed out, in slot order), each new path gets
// its camera ray (renderer.glsl:27-62) and is queued for extension in the same order (a
// depth-0 job's paths go straight to the done list with zero radiance). Handing out slots in
// slot order keeps the paths a warp shades in neighbouring slots, so their state comes in few
// cache lines, however the earlier paths finished. One scan step takes two block barriers (four
// for a multi-job pool) and one atomic per counter.
template <bool kOne>
__global__ void __launch_bounds__(kRefillBlock) engine_refill_kernel(EngineBuffers b, EngineJob one, int parity)
{
    constexpr int kG = kRefillGroups;
    constexpr int kW = kRefillBlock / 32;
    static_assert(kG * kW == 32, "one scan entry per lane of a warp");
    // double-buffered by scan step, so that a step needs no barrier at its end
    __shared__ unsigned freeMask[2][32];   // per (group, warp): free slots, then
    __shared__ int freeOff[2][32];         // their exclusive offsets in the scan step
    __shared__ int runOff[2][2][32];       // multi-job pool: queued / done offsets per (group, warp)
    __shared__ unsigned runMask[2][2][32];
    __shared__ int stepBase[2], queueBase[2], doneBase[2];
    EngineCtl* ctl = b.ctl;
    const unsigned long long next = ctl->next, total = ctl->total;
    const int freeCount = ctl->freeCount;
    const unsigned long long left = next < total ? total - next : 0ull;
    const int m = (int)((unsigned long long)freeCount < left ? (unsigned long long)freeCount : left);
    if (m <= 0) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->taken = m;
    const unsigned long long plo = ctl->passLo, phi = ctl->numPasses;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const int* infoW = reinterpret_cast<const int*>(b.ps.info) + 3;
    constexpr int kRound = kG * kRefillBlock;
    int buf = 0;
    for (int base = blockIdx.x * kRound; base < b.cap; base += gridDim.x * kRound, buf ^= 1)   // block-uniform
    {
        bool isFree[kG];
#pragma unroll
        for (int g = 0; g < kG; ++g)
        {
            const int cand = base + g * kRefillBlock + threadIdx.x;
            isFree[g] = cand < b.cap && infoW[4 * (size_t)cand] == -1;
        }
#pragma unroll
        for (int g = 0; g < kG; ++g)
        {
            const unsigned fm = __ballot_sync(kFull, isFree[g]);
            if (lane == 0) freeMask[buf][g * kW + warp] = fm;
        }
        __syncthreads();
        if (warp == 0)
        {
            int off = __popc(freeMask[buf][lane]);
            const int tot = warp_exclusive_scan(off);
            freeOff[buf][lane] = off;
            if (lane == 0)
            {
                // ids handed out so far: the share of this block's scan step, or a look at the counter
                const int rb = atomicAdd(&ctl->refillNext, tot);
                stepBase[buf] = rb;
                if constexpr (kOne)
                {
                    const int got = rb < m ? (tot < m - rb ? tot : m - rb) : 0;
                    if (got)
                        queueBase[buf] = atomicAdd(one.P.maxDepth > 0 ? &ctl->count[parity] : &ctl->doneCount[parity ^ 1],
                                                   got);
                }
            }
        }
        __syncthreads();
        const int rb = stepBase[buf];
        if (rb >= m) break;   // every id of this step is handed out
        int slotOf[kG];
        unsigned runBits = 0;
#pragma unroll 1
        for (int g = 0; g < kG; ++g)
        {
            slotOf[g] = -1;
            const unsigned fm = freeMask[buf][g * kW + warp];
            const int r = freeOff[buf][g * kW + warp] + __popc(fm & below);   // rank in the scan step
            const int k = rb + r;
            if (((fm >> lane) & 1u) && k < m)
            {
                const int slot = base + g * kRefillBlock + threadIdx.x;
                const unsigned long long id = next + (unsigned long long)k;
                const unsigned long long gp = find_pass(b.passes, id, plo, phi);
                const int ring = (int)(gp & (kPassRing - 1));
                const EnginePass& Q = b.passes[ring];
                const Params& P = kOne ? one.P : b.jobs[Q.job].P;
                const int local = (int)(id - Q.pathBase);   // passes hold < 2^31 paths
                const int visPix = Q.visW * Q.visH;
                const int s = local / visPix;
                const int lp = local - s * visPix;
                int lx, ly;
                pixel_of(lp, Q.visW, Q.visH, lx, ly);
                b.ps.L[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
                // x: the path's entry of the pass's [sample][visible pixel] radiance
                b.ps.info[slot] = make_int4(s * visPix + ly * Q.visW + lx, 0, 0, ring | (Q.job << kPassRingBits));
                gen_path(P, Q.tileX, Q.tileY, Q.tileOrdinal, Q.firstSample + s, lx, ly, b.ps, slot);
                if constexpr (kOne)
                {
                    // a single job's paths all go one way, in rank order
                    int* dst = one.P.maxDepth > 0 ? b.queue[parity] : b.done[parity ^ 1];
                    const int pos = queueBase[buf] + r;
                    if (pos < b.cap) dst[pos] = slot;
                    else set_error(b.status, LF_DEVERR_QUEUE);
                }
                else
                {
                    slotOf[g] = slot;
                    if (P.maxDepth > 0) runBits |= 1u << g;
                }
            }
        }
        if constexpr (!kOne)
        {
            // jobs of different depths: queued and done paths ranked in slot order
#pragma unroll
            for (int g = 0; g < kG; ++g)
            {
                const unsigned qm = __ballot_sync(kFull, slotOf[g] >= 0 && ((runBits >> g) & 1u));
                const unsigned dm = __ballot_sync(kFull, slotOf[g] >= 0 && !((runBits >> g) & 1u));
                if (lane == 0)
                {
                    runMask[buf][0][g * kW + warp] = qm;
                    runMask[buf][1][g * kW + warp] = dm;
                }
            }
            __syncthreads();
            if (warp == 0)
            {
                int qo = __popc(runMask[buf][0][lane]), dn = __popc(runMask[buf][1][lane]);
                const int qt = warp_exclusive_scan(qo), dt = warp_exclusive_scan(dn);
                runOff[buf][0][lane] = qo;
                runOff[buf][1][lane] = dn;
                if (lane == 0)
                {
                    queueBase[buf] = qt ? atomicAdd(&ctl->count[parity], qt) : 0;
                    doneBase[buf] = dt ? atomicAdd(&ctl->doneCount[parity ^ 1], dt) : 0;
                }
            }
            __syncthreads();
#pragma unroll
            for (int g = 0; g < kG; ++g)
            {
                if (slotOf[g] < 0) continue;
                const int q = ((runBits >> g) & 1u) ? 0 : 1;
                const int e = g * kW + warp;
                const int pos = (q ? doneBase[buf] : queueBase[buf]) + runOff[buf][q][e] +
                                __popc(runMask[buf][q][e] & below);
                int* dst = q ? b.done[parity ^ 1] : b.queue[parity];
                if (pos < b.cap) dst[pos] = slotOf[g];
                else set_error(b.status, LF_DEVERR_QUEUE);
            }
        }
    }
}

// ------------------------------------------------------------------ extend / shade / shadow
// The traversal kernels are held to 72 registers (7 blocks of 128 threads per SM; a few spills)
// whatever block size they are launched with.
template <bool kOne>
__global__ void __maxnreg__(72) engine_extend_kernel(EngineBuffers b, EngineJob one, int parity)
{
    const int n = b.ctl->count[parity];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&b.ctr[1], (unsigned long long)n);
    const int* q = b.queue[parity];
    const int lane = threadIdx.x & 31;
    while (true)
    {
        // warps take queue entries 32 at a time, so long rays do not hold up a fixed share
        int base = 0;
        if (lane == 0) base = atomicAdd(&b.ctl->extendNext, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const int i = base + lane;
        int p = -1;
        bool miss = false;
        int cls = 0;
        if (i < n)
        {
            p = q[i];
            const float4 o4 = b.ps.o[p], d4 = b.ps.d[p];
            Hit h;
            uint32_t err;
            const ShadeInstance* sinst;
            if constexpr (kOne)
            {
                err = closest_hit<false>(one.S.trav, f3(o4), f3(d4), kInfinity, one.P.useLights != 0, &h, nullptr);
                sinst = one.S.inst;
            }
            else
            {
                const int w = reinterpret_cast<const int*>(b.ps.info)[4 * p + 3];
                const EngineJob& J = b.jobs[job_of(w)];
                const DevScene T = J.S.trav;
                err = closest_hit<false>(T, f3(o4), f3(d4), kInfinity, J.P.useLights != 0, &h, nullptr);
                sinst = J.S.inst;
            }
            b.ps.hit[p] = make_float4(h.t, __int_as_float(h.inst), __int_as_float(h.prim), __int_as_float(h.light));
            set_error(b.status, err);
            miss = h.t == kInfinity;   // the shade kernel's environment case
            if (b.sortByMaterial && !miss && h.inst >= 0) cls = sinst[h.inst].shadeClass & 3;
        }
        if (b.sortByMaterial)
        {
            // hits go to the bucket of their material class, misses to the back of `part`
            const unsigned below = (1u << lane) - 1u;
#pragma unroll
            for (int k = 0; k < 4; ++k)
            {
                const unsigned km = __ballot_sync(kFull, p >= 0 && !miss && cls == k);
                int kb = 0;
                if (lane == 0 && km) kb = atomicAdd(&b.ctl->bucketCount[k], __popc(km));
                kb = __shfl_sync(kFull, kb, 0);
                if (p >= 0 && !miss && cls == k) b.partSort[(size_t)k * b.cap + kb + __popc(km & below)] = p;
            }
            const unsigned hm = __ballot_sync(kFull, p >= 0 && !miss), mm = __ballot_sync(kFull, p >= 0 && miss);
            int mb = 0;
            if (lane == 0)
            {
                if (hm) atomicAdd(&b.ctl->hitCount, __popc(hm));
                if (mm) mb = atomicAdd(&b.ctl->missCount, __popc(mm));
            }
            mb = __shfl_sync(kFull, mb, 0);
            if (p >= 0 && miss) b.part[b.cap - 1 - (mb + __popc(mm & below))] = p;
            continue;
        }
        // hits count up from the front of `part`, misses down from the back; together they
        // are the n queued paths, so the two ranges never meet
        const unsigned hm = __ballot_sync(kFull, p >= 0 && !miss), mm = __ballot_sync(kFull, p >= 0 && miss);
        int hb = 0, mb = 0;
        if (lane == 0)
        {
            if (hm) hb = atomicAdd(&b.ctl->hitCount, __popc(hm));
            if (mm) mb = atomicAdd(&b.ctl->missCount, __popc(mm));
        }
        hb = __shfl_sync(kFull, hb, 0);
        mb = __shfl_sync(kFull, mb, 0);
        const unsigned below = (1u << lane) - 1u;
        if (p >= 0 && !miss) b.part[hb + __popc(hm & below)] = p;
        if (p >= 0 && miss) b.part[b.cap - 1 - (mb + __popc(mm & below))] = p;
    }
}

// Blocks of at most 256 threads. kThreadsPerSm > 0 caps registers so that many threads fit on
// an SM (512: 128 registers, no spills; 768: 85 registers, a few spills; 1024: 64 registers);
// 0 leaves the compiler's choice.
// kLights = false: the job's scene has no analytic lights (single-job steps only).
template <bool kOne, int kThreadsPerSm, bool kLights = true>
__global__ void __launch_bounds__(256, kThreadsPerSm ? kThreadsPerSm / 256 : 1)
    engine_shade_kernel(EngineBuffers b, EngineJob one, int parity)
{
    __shared__ BlockDone bd;
    block_done_begin(bd);
    ThreadDone td;
    EngineCtl* ctl = b.ctl;
    const int n = ctl->count[parity];
    const int nHit = ctl->hitCount;   // part: hits at [0, nHit), misses at the back
    int* qout = b.queue[parity ^ 1];
    const int lane = threadIdx.x & 31;
    while (true)
    {
        // warps take 32 queue entries at a time and append their outputs with one atomic per
        // queue, so no warp waits for the others of its block
        int base = 0;
        if (lane == 0) base = atomicAdd(&ctl->shadeNext, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const int i = base + lane;
        bool pushExt = false, pushShadow = false;
        int p = -1;
        ShadowRec rec;
        if (i < n)
        {
            if (i >= nHit)
                p = b.part[b.cap - 1 - (i - nHit)];
            else if (!b.sortByMaterial)
                p = b.part[i];
            else
            {
                // hits class by class: find the bucket of position i
                int k = 0, off = i;
                while (k < 3 && off >= ctl->bucketCount[k]) off -= ctl->bucketCount[k++];
                p = b.partSort[(size_t)k * b.cap + off];
            }
            if constexpr (kOne)
                shade_path<kLights>(one.S, one.P, b.ps, p, b.ctr, pushExt, pushShadow, rec);
            else
            {
                const int w = reinterpret_cast<const int*>(b.ps.info)[4 * p + 3];
                const EngineJob& J = b.jobs[job_of(w)];
                shade_path(J.S, J.P, b.ps, p, b.ctr, pushExt, pushShadow, rec);
            }
            // a path that ends here is written out now, or by the shadow kernel after its
            // next-event rays
            if (!pushExt && pushShadow) rec.b.w = __uint_as_float(__float_as_uint(rec.b.w) | 4u);
            else if (!pushExt) end_path(b, p, b.ps.info[p], b.ps.L[p], td, bd);
        }
        __syncwarp();
        warp_push(pushExt, p, qout, &ctl->count[parity ^ 1], b.cap, b.status);
        if constexpr (kLights)
            warp_push(pushShadow, rec, b.shadow, &ctl->shadowCount, b.cap, b.status);
        else
        {
            // no light rays: the record's light fields are never read, so they are not written
            const unsigned m = __ballot_sync(kFull, pushShadow);
            if (m)
            {
                int base = 0;
                if (lane == __ffs(m) - 1) base = atomicAdd(&ctl->shadowCount, __popc(m));
                base = __shfl_sync(kFull, base, __ffs(m) - 1);
                if (pushShadow)
                {
                    const int pos = base + __popc(m & ((1u << lane) - 1u));
                    if (pos < b.cap)
                    {
                        ShadowRec* r = b.shadow + pos;
                        r->a = rec.a;
                        r->b = rec.b;
                        r->c = rec.c;
                        r->e = rec.e;
                    }
                    else
                        set_error(b.status, LF_DEVERR_QUEUE);
                }
            }
        }
    }
    block_done_end(b, td, bd);
}

template <bool kOne>
__global__ void __maxnreg__(72) engine_shadow_kernel(EngineBuffers b, EngineJob one)
{
    __shared__ BlockDone bd;
    block_done_begin(bd);
    ThreadDone td;
    const int n = b.ctl->shadowCount;
    unsigned long long rays = 0;
    const int lane = threadIdx.x & 31;
    while (true)
    {
        int base = 0;
        if (lane == 0) base = atomicAdd(&b.ctl->shadowNext, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const int i = base + lane;
        if (i >= n) continue;
        const ShadowRec* rec = b.shadow + i;
        float4 L;
        if constexpr (kOne)
            set_error(b.status, shadow_path(one.S, one.P, b.ps, rec, rays, &L));
        else
        {
            const int p = __float_as_int(rec->a.w);
            const int w = reinterpret_cast<const int*>(b.ps.info)[4 * p + 3];
            const EngineJob& J = b.jobs[job_of(w)];
            set_error(b.status, shadow_path(J.S, J.P, b.ps, rec, rays, &L));
        }
        if (__float_as_uint(rec->b.w) & 4u)   // the path ended at this record's vertex
        {
            const int p = __float_as_int(rec->a.w);
            end_path(b, p, b.ps.info[p], L, td, bd);
        }
    }
    warp_count_add(&b.ctr[2], rays);
    block_done_end(b, td, bd);
}

// ------------------------------------------------------------------ drain
// The last paths of a run, once no ids are left to issue: every queued path is taken through
// its remaining bounces by one thread (extension, shade, next-event rays, in the order of the
// step kernels) and written out. Per path this is the same sequence of operations the step
// kernels perform, so results and ray counts are unchanged; what goes away is one launch
// sequence per bounce whose length is set by the slowest ray of an almost empty pool.
// One path from its queued extension ray to its end; returns the extension and shadow rays
// it traced.
__device__ __forceinline__ void drain_path(const EngineBuffers& b, const EngineJob& J, int p, unsigned long long& ext,
                                           unsigned long long& shadowRays)
{
    for (int bounce = 0; bounce < 4096; ++bounce)
    {
        const float4 o4 = b.ps.o[p], d4 = b.ps.d[p];
        Hit h;
        const uint32_t err = closest_hit<false>(J.S.trav, f3(o4), f3(d4), kInfinity, J.P.useLights != 0, &h, nullptr);
        b.ps.hit[p] = make_float4(h.t, __int_as_float(h.inst), __int_as_float(h.prim), __int_as_float(h.light));
        set_error(b.status, err);
        ++ext;
        bool pushExt = false, pushShadow = false;
        ShadowRec rec;
        shade_path(J.S, J.P, b.ps, p, b.ctr, pushExt, pushShadow, rec);
        if (pushShadow) set_error(b.status, shadow_path(J.S, J.P, b.ps, &rec, shadowRays));
        if (!pushExt) return;
    }
}

template <bool kOne>
__global__ void __launch_bounds__(128) engine_drain_kernel(EngineBuffers b, EngineJob one, int parity)
{
    __shared__ BlockDone bd;
    block_done_begin(bd);
    ThreadDone td;
    EngineCtl* ctl = b.ctl;
    const int n = ctl->count[parity];
    const int* q = b.queue[parity];
    const int lane = threadIdx.x & 31;
    unsigned long long ext = 0, shadowRays = 0;
    while (true)
    {
        int base = 0;
        if (lane == 0) base = atomicAdd(&ctl->extendNext, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const int i = base + lane;
        if (i < n)
        {
            const int p = q[i];
            if constexpr (kOne)
                drain_path(b, one, p, ext, shadowRays);
            else
                drain_path(b, b.jobs[job_of(reinterpret_cast<const int*>(b.ps.info)[4 * p + 3])], p, ext, shadowRays);
            end_path(b, p, b.ps.info[p], b.ps.L[p], td, bd);
        }
    }
    warp_count_add(&b.ctr[1], ext);
    warp_count_add(&b.ctr[2], shadowRays);
    block_done_end(b, td, bd);
}

// ------------------------------------------------------------------ accumulate
__global__ void engine_accumulate_kernel(int width, int tileW, int tileH, EnginePass Q, float4* accum, double* accum64)
{
    const int visPix = Q.visW * Q.visH;
    for (int lp = blockIdx.x * blockDim.x + threadIdx.x; lp < visPix; lp += gridDim.x * blockDim.x)
    {
        const int lx = lp % Q.visW, ly = lp / Q.visW;
        const int gpix = (Q.tileY * tileH + ly) * width + Q.tileX * tileW + lx;
        float4 a = accum[gpix];
        double ax = 0, ay = 0, az = 0;
        if (accum64)
        {
            ax = accum64[gpix * 3 + 0];
            ay = accum64[gpix * 3 + 1];
            az = accum64[gpix * 3 + 2];
        }
        for (int s = 0; s < Q.nSamples; ++s)
        {
            const float4 l = Q.radiance[(size_t)s * visPix + lp];
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

// ------------------------------------------------------------------ launchers
namespace
{
int sm_count()
{
    static int n = 0;
    if (n == 0)
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

int full_grid(const void* kernel, int block, long long work)
{
    const int per_sm = occupancy_blocks_per_sm(kernel, block);
    long long full = (long long)sm_count() * per_sm;
    long long need = (work + block - 1) / block;
    if (need < 1) need = 1;
    return (int)(need < full ? need : full);
}
}

int launch_engine_init(const EngineBuffers& b, cudaStream_t st)
{
    engine_init_kernel<<<full_grid((const void*)engine_init_kernel, 256, b.cap), 256, 0, st>>>(b);
    return (int)cudaGetLastError();
}

int launch_engine_append(const EngineBuffers& b, unsigned long long total, unsigned long long numPasses,
                         cudaStream_t st)
{
    engine_append_kernel<<<1, 1, 0, st>>>(b, total, numPasses);
    return (int)cudaGetLastError();
}

namespace
{
template <bool kOne>
void step(const EngineBuffers& b, const EngineJob& one, int parity, cudaStream_t st)
{
    const int BF = 256;
    engine_finish_kernel<<<full_grid((const void*)engine_finish_kernel, BF, b.cap), BF, 0, st>>>(b, parity);
    engine_refill_kernel<kOne><<<full_grid((const void*)engine_refill_kernel<kOne>, kRefillBlock,
                                           (long long)b.cap / kRefillGroups),
                                 kRefillBlock, 0, st>>>(b, one, parity);
    engine_reset_kernel<<<1, 1, 0, st>>>(b.ctl, parity);
    const int be = b.blockExtend > 0 ? b.blockExtend : 128;
    const int bs = b.blockShade > 0 ? b.blockShade : 128;
    const int bw = b.blockShadow > 0 ? b.blockShadow : 128;
    engine_extend_kernel<kOne><<<full_grid((const void*)engine_extend_kernel<kOne>, be, b.cap), be, 0, st>>>(b, one,
                                                                                                           parity);
    if (b.shadeThreadsPerSm == 512 && kOne && !one.P.useLights)
        engine_shade_kernel<kOne, 512, false><<<full_grid((const void*)engine_shade_kernel<kOne, 512, false>, bs, b.cap),
                                                bs, 0, st>>>(b, one, parity);
    else if (b.shadeThreadsPerSm == 512)
        engine_shade_kernel<kOne, 512><<<full_grid((const void*)engine_shade_kernel<kOne, 512>, bs, b.cap), bs, 0, st>>>(
            b, one, parity);
    else if (b.shadeThreadsPerSm == 768)
        engine_shade_kernel<kOne, 768><<<full_grid((const void*)engine_shade_kernel<kOne, 768>, bs, b.cap), bs, 0, st>>>(
            b, one, parity);
    else if (b.shadeThreadsPerSm == 1024 && kOne && !one.P.useLights)
        engine_shade_kernel<kOne, 1024, false><<<full_grid((const void*)engine_shade_kernel<kOne, 1024, false>, bs, b.cap),
                                                 bs, 0, st>>>(b, one, parity);
    else if (b.shadeThreadsPerSm == 1024)
        engine_shade_kernel<kOne, 1024><<<full_grid((const void*)engine_shade_kernel<kOne, 1024>, bs, b.cap), bs, 0,
                                          st>>>(b, one, parity);
    else
        engine_shade_kernel<kOne, 0><<<full_grid((const void*)engine_shade_kernel<kOne, 0>, bs, b.cap), bs, 0, st>>>(
            b, one, parity);
    engine_shadow_kernel<kOne><<<full_grid((const void*)engine_shadow_kernel<kOne>, bw, b.cap), bw, 0, st>>>(b, one);
}
}

template <bool kOne>
void drain_step(const EngineBuffers& b, const EngineJob& one, cudaStream_t st)
{
    const int BF = 256;
    for (int parity = 0; parity < 2; ++parity)
    {
        engine_finish_kernel<<<full_grid((const void*)engine_finish_kernel, BF, b.cap), BF, 0, st>>>(b, parity);
        engine_refill_kernel<kOne><<<full_grid((const void*)engine_refill_kernel<kOne>, kRefillBlock,
                                               (long long)b.cap / kRefillGroups),
                                     kRefillBlock, 0, st>>>(b, one, parity);
        engine_reset_kernel<<<1, 1, 0, st>>>(b.ctl, parity);
        engine_drain_kernel<kOne><<<full_grid((const void*)engine_drain_kernel<kOne>, 128, b.cap), 128, 0, st>>>(
            b, one, parity);
    }
}

int launch_engine_drain(const EngineBuffers& b, const EngineJob* one, cudaStream_t st)
{
    if (one)
        drain_step<true>(b, *one, st);
    else
        drain_step<false>(b, EngineJob{}, st);
    return (int)cudaGetLastError();
}

int launch_engine_step(const EngineBuffers& b, const EngineJob* one, int parity, cudaStream_t st)
{
    if (one)
        step<true>(b, *one, parity, st);
    else
        step<false>(b, EngineJob{}, parity, st);
    return (int)cudaGetLastError();
}

int launch_engine_accumulate(const Params& P, const EnginePass& pass, float4* accum, double* accum64,
                             cudaStream_t st)
{
    const int B = 256;
    const long long pix = (long long)pass.visW * pass.visH;
    engine_accumulate_kernel<<<full_grid((const void*)engine_accumulate_kernel, B, pix), B, 0, st>>>(
        P.width, P.tileW, P.tileH, pass, accum, accum64);
    return (int)cudaGetLastError();
}
}
