// Host driver of the multi-job engine (device side in lf_engine.cu): pool allocation, job and
// pass tables, the graph-captured step pair and the drain loop, plus the frame renderer that
// runs lf_frame_render on it.
#include <algorithm>
#include <cstring>

#include "lf_engine.h"
#include "lf_engine_host.h"

namespace lfrt
{
namespace
{
constexpr int kDefaultSlots = 1 << 24;      // ~4.6 GB of path state (2^23 measured 2-3 % slower on C3)
constexpr int kDefaultShadeCap = 512;       // shade kernel register cap (threads per SM)
constexpr int kMaxJobs = 4096;
constexpr size_t kRunRadianceBytes = size_t(2) << 30;   // radiance buffers of one frame run

void drop_graphs(EngineHost* e)
{
    for (auto& g : e->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    e->graphs.clear();
}

void free_engine_buffers(EngineHost* e)
{
    drop_graphs(e);
    for (void* p : e->allocs) cudaFree(p);
    e->allocs.clear();
    e->b.partSort = nullptr;
}

lf_status alloc_pool(EngineHost* e, int slots)
{
    lf_ctx* c = e->c;
    size_t bytes = 0;
    cudaError_t err = cudaSuccess;
    auto A = [&](auto** p, size_t n) {
        if (err == cudaSuccess) err = dalloc(e->allocs, bytes, p, n);
    };
    EngineBuffers& b = e->b;
    A(&b.ps.o, slots);
    A(&b.ps.d, slots);
    A(&b.ps.T, slots);
    A(&b.ps.L, slots);
    A(&b.ps.A, slots);
    A(&b.ps.rng, slots);
    A(&b.ps.info, slots);
    A(&b.ps.luv, slots);
    A(&b.ps.hit, slots);
    A(&b.queue[0], slots);
    A(&b.queue[1], slots);
    A(&b.part, slots);
    A(&b.done[0], slots);
    A(&b.done[1], slots);
    A(&b.shadow, slots);
    if (e->sortMode == 1) A(&b.partSort, (size_t)4 * slots);
    if (err != cudaSuccess)
    {
        free_engine_buffers(e);
        return cuda_fail(c, err, "engine pool allocation");
    }
    b.cap = slots;
    e->poolBytes = bytes;
    return LF_OK;
}
}

lf_status engine_get(lf_ctx* c, EngineHost** out)
{
    *out = c->engine;
    if (c->engine) return LF_OK;
    EngineHost* e = new EngineHost;
    e->c = c;
    size_t bytes = 0;
    cudaError_t err = cudaSuccess;
    auto A = [&](auto** p, size_t n) {
        if (err == cudaSuccess) err = dalloc(e->tables, bytes, p, n);
    };
    EngineJob* jobs = nullptr;
    EnginePass* passes = nullptr;
    A(&jobs, kMaxJobs);
    A(&passes, kPassRing);
    A(&e->b.passDone, kPassRing);
    A(&e->b.ctl, 1);
    A(&e->ownCtr, 4);
    if (err == cudaSuccess) err = cudaMallocHost((void**)&e->h_jobStage, sizeof(EngineJob) * kMaxJobs);
    if (err == cudaSuccess) err = cudaMallocHost((void**)&e->h_passStage, sizeof(EnginePass) * kPassRing);
    for (int k = 0; k < 2 && err == cudaSuccess; ++k)
    {
        err = cudaMallocHost((void**)&e->h_ctl[k], sizeof(EngineCtl));
        if (err == cudaSuccess) err = cudaMallocHost((void**)&e->h_passDone[k], sizeof(unsigned long long) * kPassRing);
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&e->ev[k], cudaEventDisableTiming);
    }
    if (err != cudaSuccess)
    {
        engine_destroy(e);
        return cuda_fail(c, err, "engine table allocation");
    }
    e->b.jobs = jobs;
    e->b.passes = passes;
    e->b.status = c->d_status;
    e->b.ctr = e->ownCtr;
    e->b.shadeThreadsPerSm = kDefaultShadeCap;
    e->jobUsed.assign(kMaxJobs, 0);
    e->jobGen.assign(kMaxJobs, 0);
    // pass radiance buffers come from the stream-ordered pool; keep up to 8 GB of it cached
    // between runs instead of handing it back to CUDA at every synchronisation
    cudaMemPool_t pool = nullptr;
    if (cudaDeviceGetDefaultMemPool(&pool, c->device) == cudaSuccess)
    {
        uint64_t keep = uint64_t(8) << 30;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaMemsetAsync(e->b.ctl, 0, sizeof(EngineCtl), c->stream);
    cudaMemsetAsync(e->b.passDone, 0, sizeof(unsigned long long) * kPassRing, c->stream);
    cudaMemsetAsync(e->ownCtr, 0, 4 * sizeof(unsigned long long), c->stream);
    lf_status st = alloc_pool(e, kDefaultSlots);
    if (st == LF_OK && launch_engine_init(e->b, c->stream) != 0) st = fail(c, LF_ERR_CUDA, "engine init launch");
    if (st != LF_OK)
    {
        engine_destroy(e);
        return st;
    }
    c->engine = e;
    *out = e;
    return LF_OK;
}

void engine_destroy(EngineHost* e)
{
    if (!e) return;
    if (e->c && e->c->stream) cudaStreamSynchronize(e->c->stream);
    free_engine_buffers(e);
    for (void* p : e->tables) cudaFree(p);
    if (e->h_jobStage) cudaFreeHost(e->h_jobStage);
    if (e->h_passStage) cudaFreeHost(e->h_passStage);
    for (int k = 0; k < 2; ++k)
    {
        if (e->h_ctl[k]) cudaFreeHost(e->h_ctl[k]);
        if (e->h_passDone[k]) cudaFreeHost(e->h_passDone[k]);
        if (e->ev[k]) cudaEventDestroy(e->ev[k]);
    }
    delete e;
}

lf_status engine_configure(EngineHost* e, int slots, int blockExtend, int blockShade, int blockShadow,
                           int shadeThreadsPerSm)
{
    lf_ctx* c = e->c;
    auto okBlock = [](int b) { return b == 0 || (b >= 32 && b <= 1024 && b % 32 == 0); };
    const bool capOk = (shadeThreadsPerSm == 0 || shadeThreadsPerSm == 512 || shadeThreadsPerSm == 768 ||
                        shadeThreadsPerSm == 1024) &&
                       blockShade <= 256;
    if (slots < 0 || !okBlock(blockExtend) || !okBlock(blockShade) || !okBlock(blockShadow) || !capOk)
        return fail(c, LF_ERR_INVALID, "engine configuration out of range");
    if (e->active > 0) return fail(c, LF_ERR_STATE, "engine has passes in flight");
    cudaStreamSynchronize(c->stream);
    e->b.blockExtend = blockExtend;
    e->b.blockShade = blockShade;
    e->b.blockShadow = blockShadow;
    e->b.shadeThreadsPerSm = shadeThreadsPerSm;
    drop_graphs(e);
    if (slots > 0 && slots != e->b.cap)
    {
        free_engine_buffers(e);
        lf_status st = alloc_pool(e, slots);
        if (st != LF_OK) return st;
        if (launch_engine_init(e->b, c->stream) != 0) return fail(c, LF_ERR_CUDA, "engine init launch");
    }
    return LF_OK;
}

namespace
{
lf_status ensure_sort_buckets(EngineHost* e)
{
    if (e->b.partSort) return LF_OK;
    size_t bytes = 0;
    cudaError_t err = dalloc(e->allocs, bytes, &e->b.partSort, (size_t)4 * e->b.cap);
    if (err != cudaSuccess) return cuda_fail(e->c, err, "sort-by-material buckets");
    e->poolBytes += bytes;
    return LF_OK;
}

// Whether the steps of `one` (nullptr: the multi-job form) sort by material.
bool sort_on(const EngineHost* e, const EngineJob* one)
{
    if (e->sortMode == 1) return true;
    if (e->sortMode == 0 || !one) return false;
    const uint32_t m = one->S.shadeClassMask;
    return (m & (m - 1)) != 0;   // more than one class
}
}

lf_status engine_set_sort(EngineHost* e, int mode)
{
    lf_ctx* c = e->c;
    if (e->active > 0) return fail(c, LF_ERR_STATE, "engine has passes in flight");
    cudaStreamSynchronize(c->stream);
    if (mode == 1)
    {
        lf_status st = ensure_sort_buckets(e);
        if (st != LF_OK) return st;
    }
    e->sortMode = mode;
    drop_graphs(e);   // the graphs hold the kernel parameters
    return LF_OK;
}

int engine_job_alloc(EngineHost* e, const ShadeScene& S, const Params& P)
{
    for (int j = 0; j < kMaxJobs; ++j)
        if (!e->jobUsed[j])
        {
            e->jobUsed[j] = 1;
            engine_job_write(e, j, S, P);
            return j;
        }
    return -1;
}

void engine_job_write(EngineHost* e, int j, const ShadeScene& S, const Params& P)
{
    EngineJob J;
    std::memset(&J, 0, sizeof J);
    std::memcpy(&J.S, &S, sizeof S);
    J.S.env.multiplier = P.hdrMultiplier;
    std::memcpy(&J.P, &P, sizeof P);
    if (std::memcmp(&J, &e->h_jobStage[j], sizeof J) == 0 && e->jobGen[j] != 0) return;
    // the staging entry is only rewritten once earlier copies from it have executed
    cudaStreamSynchronize(e->c->stream);
    std::memcpy(&e->h_jobStage[j], &J, sizeof J);
    ++e->jobGen[j];
    cudaMemcpyAsync((void*)(e->b.jobs + j), &e->h_jobStage[j], sizeof(EngineJob), cudaMemcpyHostToDevice,
                    e->c->stream);
}

void engine_job_free(EngineHost* e, int j)
{
    if (j >= 0 && j < kMaxJobs) e->jobUsed[j] = 0;
}

unsigned long long engine_pass_submit(EngineHost* e, EnginePass desc)
{
    const unsigned long long g = e->numPasses++;
    const int r = (int)(g & (kPassRing - 1));
    desc.pathBase = e->total;
    e->total += desc.numPaths;
    e->h_passStage[r] = desc;
    cudaMemcpyAsync((void*)(e->b.passes + r), &e->h_passStage[r], sizeof(EnginePass), cudaMemcpyHostToDevice,
                    e->c->stream);
    cudaMemsetAsync(e->b.passDone + r, 0, sizeof(unsigned long long), e->c->stream);
    ++e->active;
    return g;
}

lf_status engine_publish(EngineHost* e)
{
    if (launch_engine_append(e->b, e->total, e->numPasses, e->c->stream) != 0)
        return fail(e->c, LF_ERR_CUDA, "engine append launch");
    return LF_OK;
}

lf_status engine_launch_pair(EngineHost* e, unsigned long long* ctr, int job, bool drain)
{
    lf_ctx* c = e->c;
    if (!ctr) ctr = e->ownCtr;
    const unsigned gen = job >= 0 ? e->jobGen[job] : 0;
    EngineHost::Graph* hit = nullptr;
    for (auto& g : e->graphs)
        if (g.ctr == ctr && g.job == job && g.gen == gen && g.drain == drain) hit = &g;
    if (!hit)
    {
        if (e->graphs.size() >= 8) drop_graphs(e);
        const EngineJob* one = job >= 0 ? &e->h_jobStage[job] : nullptr;
        const bool sort = sort_on(e, one);
        if (sort)
        {
            lf_status st = ensure_sort_buckets(e);
            if (st != LF_OK) return st;
        }
        EngineBuffers b = e->b;
        b.ctr = ctr;
        b.sortByMaterial = sort ? 1 : 0;
        cudaGraph_t g = nullptr;
        cudaGraphExec_t exec = nullptr;
        cudaError_t err = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
        if (err != cudaSuccess) return cuda_fail(c, err, "engine graph capture");
        int le = 0;
        if (drain)
            le = launch_engine_drain(b, one, c->stream);
        else
        {
            le = launch_engine_step(b, one, 0, c->stream);
            le |= launch_engine_step(b, one, 1, c->stream);
        }
        err = cudaStreamEndCapture(c->stream, &g);
        if (err == cudaSuccess && le) err = (cudaError_t)le;
        if (err == cudaSuccess) err = cudaGraphInstantiate(&exec, g, 0);
        if (g) cudaGraphDestroy(g);
        if (err != cudaSuccess) return cuda_fail(c, err, "engine graph instantiate");
        e->graphs.push_back({exec, ctr, job, gen, drain});
        hit = &e->graphs.back();
    }
    cudaError_t err = cudaGraphLaunch(hit->exec, c->stream);
    if (err != cudaSuccess) return cuda_fail(c, err, "engine graph launch");
    return LF_OK;
}

lf_status engine_snapshot(EngineHost* e, int k)
{
    lf_ctx* c = e->c;
    cudaMemcpyAsync(e->h_ctl[k], e->b.ctl, sizeof(EngineCtl), cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(e->h_passDone[k], e->b.passDone, sizeof(unsigned long long) * kPassRing, cudaMemcpyDeviceToHost,
                    c->stream);
    cudaError_t err = cudaEventRecord(e->ev[k], c->stream);
    if (err != cudaSuccess) return cuda_fail(c, err, "engine snapshot");
    return LF_OK;
}

lf_status engine_drain(EngineHost* e, unsigned long long* ctr, int maxDepth, int job)
{
    lf_ctx* c = e->c;
    // Bound on steps: every path needs at most maxDepth + 1 steps after it starts, and at
    // least `cap` paths start per step while work remains.
    const unsigned long long limit =
        8ull * ((e->total + (unsigned long long)e->b.cap - 1) / (unsigned long long)e->b.cap + 2) *
            (unsigned long long)(maxDepth + 2) + 64ull;
    unsigned long long pairs = 0;
    bool drain = false;
    lf_status st = engine_launch_pair(e, ctr, job);
    if (st == LF_OK) st = engine_snapshot(e, 0);
    int cur = 0;
    while (st == LF_OK)
    {
        st = engine_launch_pair(e, ctr, job, drain);
        if (st == LF_OK) st = engine_snapshot(e, cur ^ 1);
        if (st != LF_OK) break;
        cudaError_t err = cudaEventSynchronize(e->ev[cur]);
        if (err != cudaSuccess) return cuda_fail(c, err, "engine step");
        const EngineCtl& s = *e->h_ctl[cur];
        if (s.active == 0 && s.next >= s.total) break;
        // once every id is issued and few paths remain, run them to their ends in one kernel
        if (e->drainPaths > 0 && s.next >= s.total && s.active <= e->drainPaths) drain = true;
        if (++pairs * 2 > limit) return fail(c, LF_ERR_DEVICE, "engine did not drain");
        cur ^= 1;
    }
    if (st != LF_OK) return st;
    cudaError_t err = cudaEventSynchronize(e->ev[cur ^ 1]);
    if (err != cudaSuccess) return cuda_fail(c, err, "engine step");
    return LF_OK;
}

// ------------------------------------------------------------------ frames on the engine
lf_status frame_render_engine(lf_frame* f, const Params& Pf, int firstSample, int count)
{
    lf_ctx* c = f->ctx;
    EngineHost* e = nullptr;
    lf_status st = engine_get(c, &e);
    if (st != LF_OK) return st;
    if (f->engineJob < 0)
    {
        f->engineJob = engine_job_alloc(e, f->scene->view, Pf);
        if (f->engineJob < 0) return fail(c, LF_ERR_STATE, "engine job table full");
    }
    else
        engine_job_write(e, f->engineJob, f->scene->view, Pf);
    if (f->lastRadiance)
    {
        cudaFreeAsync(f->lastRadiance, c->stream);
        f->lastRadiance = nullptr;
        f->lastRadianceSamples = 0;
    }
    const bool tiledFrames = (f->flags & LF_FRAME_TILED_FRAMES) != 0;
    const long long tilePix = (long long)Pf.tileW * Pf.tileH;
    // samples per pass: the frame's batch size, and below 2^31 paths per pass
    const int chunk = (int)std::max(1LL, std::min<long long>(f->sppBatch, (1LL << 30) / tilePix));
    struct Pending
    {
        EnginePass desc;
    };
    std::vector<Pending> run;
    size_t runBytes = 0;
    auto flush = [&]() -> lf_status {
        if (run.empty()) return LF_OK;
        lf_status s2 = engine_publish(e);
        if (s2 == LF_OK) s2 = engine_drain(e, f->bb.ctr, Pf.maxDepth, f->engineJob);
        if (s2 != LF_OK) return s2;
        for (size_t i = 0; i < run.size(); ++i)
        {
            const EnginePass& q = run[i].desc;
            if (launch_engine_accumulate(Pf, q, f->accum, f->accum64, c->stream) != 0)
                return fail(c, LF_ERR_CUDA, "engine accumulate launch");
            const bool keep = i + 1 == run.size() && f->numTilesX * f->numTilesY == 1;
            if (keep)
            {
                f->lastRadiance = q.radiance;
                f->lastRadianceSamples = q.nSamples;
            }
            else
                cudaFreeAsync(q.radiance, c->stream);
        }
        e->active -= (long long)run.size();
        run.clear();
        runBytes = 0;
        return LF_OK;
    };
    for (int s = 0; s < count; s += chunk)
    {
        const int n = std::min(chunk, count - s);
        for (int ty = f->numTilesY - 1; ty >= 0; --ty)   // TiledRenderer order: top tile row first
            for (int tx = 0; tx < f->numTilesX; ++tx)
            {
                EnginePass q{};
                q.job = f->engineJob;
                q.firstSample = firstSample + s;
                q.nSamples = n;
                q.tileX = tx;
                q.tileY = ty;
                q.tileOrdinal = tiledFrames ? (f->numTilesY - 1 - ty) * f->numTilesX + tx : 0;
                q.visW = std::min(Pf.tileW, f->W - tx * Pf.tileW);
                q.visH = std::min(Pf.tileH, f->H - ty * Pf.tileH);
                q.numPaths = (unsigned long long)n * q.visW * q.visH;
                const size_t bytes = sizeof(float4) * q.numPaths;
                if (!run.empty() && (runBytes + bytes > kRunRadianceBytes || run.size() + 1 >= (size_t)kPassRing / 2))
                {
                    st = flush();
                    if (st != LF_OK) return st;
                }
                cudaError_t err = cudaMallocAsync((void**)&q.radiance, bytes, c->stream);
                if (err != cudaSuccess) return cuda_fail(c, err, "pass radiance allocation");
                engine_pass_submit(e, q);
                run.push_back({q});
                runBytes += bytes;
            }
    }
    return flush();
}
}
