// Serving loop: a scheduler thread that admits render jobs under a device-memory budget and
// runs the sample passes of every admitted job in the same engine launches (continuous
// batching). Scenes are uploaded on admission and stay resident while memory allows; idle
// scenes are evicted least recently used first.
//
// Per scheduler iteration:
//   1. admit queued jobs in arrival order while the budget holds them (scene upload, job
//      slot, accumulation buffer); a job that does not fit blocks the ones behind it;
//   2. give each running job up to `passes_per_job` passes in flight (about paths_per_pass
//      paths each, whole samples), publish them;
//   3. run one graph-captured pair of engine steps and read the control block back;
//   4. accumulate the passes that completed, in sample order per job; a job whose samples are
//      all accumulated is done once its last accumulation has executed (event).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <thread>

#include "lf_engine_host.h"

using namespace lfrt;

namespace
{
constexpr uint64_t kDefaultBudget = uint64_t(150) << 30;

struct ServerScene
{
    lf_scene_view view{};
    lf_scene* dev = nullptr;   // resident copy, or null
    size_t bytes = 0;          // device bytes when resident (estimate before the first upload)
    uint64_t lastUse = 0;
    int users = 0;             // queued + running jobs
    int running = 0;           // running jobs: the scene may be evicted only when none runs
};

struct ServerPass
{
    EnginePass desc{};
    unsigned long long g = 0;  // global pass index
    size_t bytes = 0;
};

struct ServerJob
{
    int64_t id = 0;
    int64_t scene = 0;
    lf_render_params params{};
    Params P{};
    int spp = 0;
    int issued = 0;            // samples handed to passes
    int accumulated = 0;
    int state = LF_JOB_QUEUED;
    int engineJob = -1;
    float4* accum = nullptr;
    size_t accumBytes = 0;
    size_t passReserve = 0;    // budget held for the job's pass buffers while it runs
    std::deque<ServerPass> inflight;
    cudaEvent_t doneEvent = nullptr;
    double submitMs = 0, startMs = 0, finishMs = 0;
};
}

struct lf_server
{
    lf_ctx* ctx = nullptr;
    EngineHost* engine = nullptr;
    lf_server_config cfg{};
    std::mutex mu;
    std::condition_variable cv;     // wakes the scheduler
    std::condition_variable doneCv; // wakes waiters
    std::thread thread;
    bool stop = false;
    std::chrono::steady_clock::time_point t0;
    std::map<int64_t, ServerScene> scenes;
    std::map<int64_t, ServerJob> jobs;
    std::deque<int64_t> queue;      // admission order
    int64_t nextScene = 1, nextJob = 1;
    uint64_t useClock = 0;
    uint64_t deviceBytes = 0;       // resident scenes + pool + job buffers
    lf_server_stats stats{};
    unsigned long long ctrBase[4] = {0, 0, 0, 0};   // engine counters at creation
    std::string err;
};

namespace
{
double now_ms(const lf_server* s)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - s->t0).count();
}

// lf_scene_upload's allocations for a view (used before the first upload): inner-node
// records (a binary tree has fewer inner nodes than half its nodes plus one), triangle
// records and indices, vertices and normals, instance records, materials, lights,
// environment tables and texture layers.
size_t estimate_scene_bytes(const lf_scene_view& v)
{
    size_t b = 0;
    b += ((size_t)v.num_nodes / 2 + 1) * 4 * sizeof(float4);
    b += (size_t)v.num_tris * (3 * sizeof(float4) + sizeof(int4));
    b += (size_t)v.num_vertices * 2 * sizeof(float4);
    b += (size_t)v.num_instances * (4 * sizeof(float4) + sizeof(ShadeInstance));
    b += (size_t)v.num_materials * sizeof(DevMaterial) + (size_t)v.num_lights * sizeof(DevLight);
    b += (size_t)v.env_width * v.env_height * (3 * sizeof(float) + sizeof(float2)) + (size_t)v.env_height * sizeof(float2);
    b += (size_t)v.num_textures * v.tex_width * v.tex_height * 4;
    return b + 4096;
}

size_t pass_paths(const lf_server* s, const ServerJob& j)
{
    (void)j;
    if (s->cfg.paths_per_pass > 0) return (size_t)s->cfg.paths_per_pass;
    return (size_t)s->engine->b.cap;
}

int pass_samples(const lf_server* s, const ServerJob& j)
{
    const size_t pix = (size_t)j.params.width * j.params.height;
    const size_t per = std::max<size_t>(1, pass_paths(s, j) / std::max<size_t>(1, pix));
    return (int)std::min<size_t>(per, (size_t)std::max(0, j.spp - j.issued));
}

size_t job_need(const lf_server* s, const ServerJob& j)
{
    const size_t pix = (size_t)j.params.width * j.params.height;
    const size_t perPass = std::max<size_t>(1, pass_paths(s, j) / std::max<size_t>(1, pix));
    const int passes = s->cfg.passes_per_job > 0 ? s->cfg.passes_per_job : 2;
    return pix * sizeof(float4) + (size_t)passes * std::min<size_t>(perPass, (size_t)j.spp) * pix * sizeof(float4);
}

// Evicts idle resident scenes (no running job; least recently used first) until `need` more
// bytes fit. A scene that only queued jobs refer to is idle: it is uploaded again when one of
// them is admitted.
bool make_room(lf_server* s, size_t need, const ServerScene* keep)
{
    const uint64_t budget = s->cfg.memory_budget;
    while (s->deviceBytes + need > budget)
    {
        ServerScene* victim = nullptr;
        for (auto& kv : s->scenes)
        {
            ServerScene& sc = kv.second;
            if (&sc != keep && sc.dev && sc.running == 0 && (!victim || sc.lastUse < victim->lastUse)) victim = &sc;
        }
        if (!victim) return false;
        lf_scene_release(victim->dev);
        victim->dev = nullptr;
        s->deviceBytes -= victim->bytes;
        s->stats.scene_evictions++;
    }
    return true;
}

// Tries to admit the job: scene resident, engine job slot, accumulation buffer.
bool admit(lf_server* s, ServerJob& j)
{
    lf_ctx* c = s->ctx;
    ServerScene& sc = s->scenes[j.scene];
    const size_t need = job_need(s, j) + (sc.dev ? 0 : sc.bytes);
    if (!make_room(s, need, &sc)) return false;
    if (!sc.dev)
    {
        lf_scene* dev = nullptr;
        if (lf_scene_upload(c, &sc.view, &dev) != LF_OK) return false;
        sc.dev = dev;
        sc.bytes = lf_scene_device_bytes(dev);
        s->deviceBytes += sc.bytes;
        s->stats.scene_uploads++;
    }
    sc.lastUse = ++s->useClock;
    fill_params(j.P, &j.params, sc.dev);
    j.engineJob = engine_job_alloc(s->engine, sc.dev->view, j.P);
    if (j.engineJob < 0) return false;
    j.accumBytes = (size_t)j.params.width * j.params.height * sizeof(float4);
    if (cudaMallocAsync((void**)&j.accum, j.accumBytes, c->stream) != cudaSuccess)
    {
        cudaGetLastError();
        engine_job_free(s->engine, j.engineJob);
        j.engineJob = -1;
        return false;
    }
    cudaMemsetAsync(j.accum, 0, j.accumBytes, c->stream);
    j.passReserve = job_need(s, j) - j.accumBytes;
    s->deviceBytes += j.accumBytes + j.passReserve;
    sc.running++;
    j.state = LF_JOB_RUNNING;
    j.startMs = now_ms(s);
    return true;
}

bool issue_passes(lf_server* s, ServerJob& j)
{
    lf_ctx* c = s->ctx;
    const int maxInflight = s->cfg.passes_per_job > 0 ? s->cfg.passes_per_job : 2;
    bool any = false;
    while ((int)j.inflight.size() < maxInflight && j.issued < j.spp)
    {
        const int n = pass_samples(s, j);
        ServerPass sp;
        EnginePass& q = sp.desc;
        q.job = j.engineJob;
        q.firstSample = j.issued;
        q.nSamples = n;
        q.tileX = q.tileY = q.tileOrdinal = 0;
        q.visW = j.params.width;
        q.visH = j.params.height;
        q.numPaths = (unsigned long long)n * q.visW * q.visH;
        sp.bytes = sizeof(float4) * q.numPaths;   // within the job's reservation
        if (cudaMallocAsync((void**)&q.radiance, sp.bytes, c->stream) != cudaSuccess)
        {
            cudaGetLastError();
            break;
        }
        sp.g = engine_pass_submit(s->engine, q);
        j.issued += n;
        j.inflight.push_back(sp);
        any = true;
    }
    return any;
}

void finish_job(lf_server* s, ServerJob& j)
{
    if (!j.doneEvent) cudaEventCreateWithFlags(&j.doneEvent, cudaEventDisableTiming);
    cudaEventRecord(j.doneEvent, s->ctx->stream);
}

void scheduler(lf_server* s)
{
    lf_ctx* c = s->ctx;
    EngineHost* e = s->engine;
    std::unique_lock<std::mutex> lk(s->mu);
    while (true)
    {
        // 1. admission in arrival order
        while (!s->queue.empty())
        {
            ServerJob& j = s->jobs[s->queue.front()];
            std::lock_guard<std::recursive_mutex> g(c->mu);
            cudaSetDevice(c->device);
            if (admit(s, j))
            {
                s->queue.pop_front();
                continue;
            }
            bool anyRunning = false;
            for (auto& kv : s->jobs)
                if (kv.second.state == LF_JOB_RUNNING) anyRunning = true;
            if (anyRunning) break;   // running jobs will free their reservations
            // Nothing runs and every idle scene is evicted, yet the job does not fit: the
            // budget is held by finished jobs whose buffers were not released. Fail the job
            // instead of waiting for memory that nothing will free.
            s->err = "job " + std::to_string(j.id) +
                     " cannot be admitted: the memory budget is held by finished jobs that were not released";
            j.state = LF_JOB_FAILED;
            j.finishMs = now_ms(s);
            s->scenes[j.scene].users--;
            s->queue.pop_front();
            s->doneCv.notify_all();
        }
        // 2. passes
        bool published = false;
        int running = 0, lastJob = -1;
        bool oneJob = true;
        {
            std::lock_guard<std::recursive_mutex> g(c->mu);
            cudaSetDevice(c->device);
            for (auto& kv : s->jobs)
            {
                ServerJob& j = kv.second;
                if (j.state != LF_JOB_RUNNING) continue;
                published |= issue_passes(s, j);
                if (!j.inflight.empty())
                {
                    ++running;
                    if (lastJob >= 0 && lastJob != j.engineJob) oneJob = false;
                    lastJob = j.engineJob;
                }
            }
            if (published) engine_publish(e);
        }
        // finished jobs waiting for their last accumulation
        for (auto& kv : s->jobs)
        {
            ServerJob& j = kv.second;
            if (j.state == LF_JOB_RUNNING && j.doneEvent && j.accumulated == j.spp &&
                cudaEventQuery(j.doneEvent) == cudaSuccess)
            {
                j.state = LF_JOB_DONE;
                j.finishMs = now_ms(s);
                s->deviceBytes -= j.passReserve;
                j.passReserve = 0;
                s->stats.jobs_done++;
                s->scenes[j.scene].users--;
                s->scenes[j.scene].running--;
                s->scenes[j.scene].lastUse = ++s->useClock;
                engine_job_free(e, j.engineJob);
                j.engineJob = -1;
                s->doneCv.notify_all();
            }
        }
        if (running == 0)
        {
            bool pending = false;
            for (auto& kv : s->jobs)
                if (kv.second.state == LF_JOB_RUNNING) pending = true;
            if (s->stop && !pending) break;
            if (!pending && s->queue.empty())
                s->cv.wait(lk);
            else
                s->cv.wait_for(lk, std::chrono::microseconds(200));
            continue;
        }
        // 3. one pair of steps (unlocked while the GPU runs)
        lk.unlock();
        lf_status st;
        {
            std::lock_guard<std::recursive_mutex> g(c->mu);
            cudaSetDevice(c->device);
            st = engine_launch_pair(e, nullptr, oneJob ? lastJob : -1);
            if (st == LF_OK) st = engine_snapshot(e, 0);
        }
        if (st == LF_OK && cudaEventSynchronize(e->ev[0]) != cudaSuccess) st = LF_ERR_CUDA;
        lk.lock();
        if (st != LF_OK)
        {
            s->err = c->err.empty() ? "engine step failed" : c->err;
            for (auto& kv : s->jobs)
                if (kv.second.state == LF_JOB_RUNNING || kv.second.state == LF_JOB_QUEUED) kv.second.state = LF_JOB_FAILED;
            s->queue.clear();
            s->doneCv.notify_all();
            break;
        }
        // 4. completed passes, in order per job
        std::lock_guard<std::recursive_mutex> g(c->mu);
        cudaSetDevice(c->device);
        for (auto& kv : s->jobs)
        {
            ServerJob& j = kv.second;
            while (!j.inflight.empty())
            {
                ServerPass& sp = j.inflight.front();
                const int r = (int)(sp.g & (kPassRing - 1));
                if (e->h_passDone[0][r] < sp.desc.numPaths) break;
                launch_engine_accumulate(j.P, sp.desc, j.accum, nullptr, c->stream);
                cudaFreeAsync(sp.desc.radiance, c->stream);
                s->stats.paths += sp.desc.numPaths;
                j.accumulated += sp.desc.nSamples;
                e->active -= 1;
                j.inflight.pop_front();
            }
            if (j.state == LF_JOB_RUNNING && j.accumulated == j.spp && !j.doneEvent) finish_job(s, j);
        }
    }
}
}

extern "C" {

lf_status lf_server_create(lf_ctx* c, const lf_server_config* cfg, lf_server** out)
{
    if (!c || !out) return LF_ERR_INVALID;
    *out = nullptr;
    lf_server* s = new lf_server;
    s->ctx = c;
    if (cfg) s->cfg = *cfg;
    if (s->cfg.memory_budget == 0) s->cfg.memory_budget = kDefaultBudget;
    if (s->cfg.paths_per_pass < 0 || s->cfg.passes_per_job < 0)
    {
        delete s;
        return fail(c, LF_ERR_INVALID, "bad server configuration");
    }
    {
        std::lock_guard<std::recursive_mutex> g(c->mu);
        cudaSetDevice(c->device);
        lf_status st = engine_get(c, &s->engine);
        if (st != LF_OK)
        {
            delete s;
            return st;
        }
    }
    s->deviceBytes = s->engine->poolBytes;
    {
        std::lock_guard<std::recursive_mutex> g(c->mu);
        cudaMemcpyAsync(s->ctrBase, s->engine->ownCtr, sizeof s->ctrBase, cudaMemcpyDeviceToHost, c->stream);
        cudaStreamSynchronize(c->stream);
    }
    if (s->deviceBytes > s->cfg.memory_budget)
    {
        delete s;
        return fail(c, LF_ERR_BUDGET, "the engine pool alone exceeds the memory budget");
    }
    s->t0 = std::chrono::steady_clock::now();
    s->thread = std::thread(scheduler, s);
    *out = s;
    return LF_OK;
}

lf_status lf_server_add_scene(lf_server* s, const lf_scene_view* v, int64_t* scene_id)
{
    if (!s || !v || !scene_id || !v->nodes || v->num_nodes <= 0) return LF_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    ServerScene sc;
    sc.view = *v;
    sc.bytes = estimate_scene_bytes(*v);
    const int64_t id = s->nextScene++;
    s->scenes[id] = sc;
    *scene_id = id;
    return LF_OK;
}

lf_status lf_server_remove_scene(lf_server* s, int64_t scene_id)
{
    if (!s) return LF_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->scenes.find(scene_id);
    if (it == s->scenes.end()) return LF_ERR_INVALID;
    if (it->second.users > 0) return fail(s->ctx, LF_ERR_STATE, "scene in use");
    if (it->second.dev)
    {
        std::lock_guard<std::recursive_mutex> g(s->ctx->mu);
        lf_scene_release(it->second.dev);
        s->deviceBytes -= it->second.bytes;
    }
    s->scenes.erase(it);
    return LF_OK;
}

lf_status lf_server_submit(lf_server* s, int64_t scene_id, const lf_render_params* p, int32_t spp, int64_t* job_id)
{
    if (!s || !p || !job_id || spp <= 0 || p->width <= 0 || p->height <= 0 || p->max_depth < 0) return LF_ERR_INVALID;
    if (p->tile_width > 0 || p->tile_height > 0) return fail(s->ctx, LF_ERR_INVALID, "server jobs render whole frames");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->scenes.find(scene_id);
    if (it == s->scenes.end()) return LF_ERR_INVALID;
    ServerJob j;
    j.id = s->nextJob++;
    j.scene = scene_id;
    j.params = *p;
    j.spp = spp;
    j.submitMs = now_ms(s);
    if (job_need(s, j) + it->second.bytes + s->engine->poolBytes > s->cfg.memory_budget)
        return fail(s->ctx, LF_ERR_BUDGET, "job does not fit the memory budget");
    it->second.users++;
    s->jobs[j.id] = j;
    s->queue.push_back(j.id);
    s->stats.jobs_submitted++;
    *job_id = j.id;
    s->cv.notify_all();
    return LF_OK;
}

lf_status lf_server_job_info(lf_server* s, int64_t job_id, lf_job_info* out)
{
    if (!s || !out) return LF_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return LF_ERR_INVALID;
    const ServerJob& j = it->second;
    out->state = j.state;
    out->samples_done = j.accumulated;
    out->submit_ms = j.submitMs;
    out->start_ms = j.startMs;
    out->finish_ms = j.finishMs;
    return LF_OK;
}

lf_status lf_server_wait(lf_server* s, int64_t job_id, int32_t timeout_ms)
{
    if (!s) return LF_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto done = [&]() {
        auto it = s->jobs.find(job_id);
        return it == s->jobs.end() || it->second.state == LF_JOB_DONE || it->second.state == LF_JOB_FAILED;
    };
    if (timeout_ms < 0)
        s->doneCv.wait(lk, done);
    else if (!s->doneCv.wait_for(lk, std::chrono::milliseconds(timeout_ms), done))
        return LF_ERR_TIMEOUT;
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return LF_ERR_INVALID;
    return it->second.state == LF_JOB_DONE ? LF_OK : fail(s->ctx, LF_ERR_DEVICE, s->err);
}

lf_status lf_server_read(lf_server* s, int64_t job_id, float* rgb)
{
    if (!s || !rgb) return LF_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return LF_ERR_INVALID;
    ServerJob& j = it->second;
    if (j.state != LF_JOB_DONE) return fail(s->ctx, LF_ERR_STATE, "job not done");
    std::vector<float4> tmp((size_t)j.params.width * j.params.height);
    lf_ctx* c = s->ctx;
    std::lock_guard<std::recursive_mutex> g(c->mu);
    cudaSetDevice(c->device);
    cudaError_t e = cudaMemcpyAsync(tmp.data(), j.accum, tmp.size() * sizeof(float4), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "job readback");
    for (size_t i = 0; i < tmp.size(); ++i)
    {
        rgb[i * 3 + 0] = tmp[i].x;
        rgb[i * 3 + 1] = tmp[i].y;
        rgb[i * 3 + 2] = tmp[i].z;
    }
    return LF_OK;
}

lf_status lf_server_release_job(lf_server* s, int64_t job_id)
{
    if (!s) return LF_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return LF_ERR_INVALID;
    ServerJob& j = it->second;
    if (j.state == LF_JOB_RUNNING) return fail(s->ctx, LF_ERR_STATE, "job running");
    if (j.state == LF_JOB_QUEUED)
    {
        s->queue.erase(std::remove(s->queue.begin(), s->queue.end(), job_id), s->queue.end());
        s->scenes[j.scene].users--;
    }
    {
        std::lock_guard<std::recursive_mutex> g(s->ctx->mu);
        cudaSetDevice(s->ctx->device);
        if (j.accum)
        {
            cudaFreeAsync(j.accum, s->ctx->stream);
            s->deviceBytes -= j.accumBytes;
        }
        if (j.doneEvent) cudaEventDestroy(j.doneEvent);
    }
    s->jobs.erase(it);
    s->cv.notify_all();
    return LF_OK;
}

lf_status lf_server_get_stats(lf_server* s, lf_server_stats* out)
{
    if (!s || !out) return LF_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    unsigned long long ctr[4] = {0, 0, 0, 0};
    {
        std::lock_guard<std::recursive_mutex> g(s->ctx->mu);
        cudaSetDevice(s->ctx->device);
        cudaMemcpyAsync(ctr, s->engine->ownCtr, sizeof ctr, cudaMemcpyDeviceToHost, s->ctx->stream);
        cudaStreamSynchronize(s->ctx->stream);
    }
    out->ext_rays = ctr[1] - s->ctrBase[1];
    out->shadow_rays = ctr[2] - s->ctrBase[2];
    out->device_bytes = s->deviceBytes;
    out->scenes_resident = 0;
    for (auto& kv : s->scenes)
        if (kv.second.dev) out->scenes_resident++;
    out->jobs_running = 0;
    for (auto& kv : s->jobs)
        if (kv.second.state == LF_JOB_RUNNING) out->jobs_running++;
    out->jobs_queued = (int32_t)s->queue.size();
    return LF_OK;
}

lf_status lf_server_destroy(lf_server* s)
{
    if (!s) return LF_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (int64_t id : s->queue)
        {
            s->jobs[id].state = LF_JOB_FAILED;
            s->scenes[s->jobs[id].scene].users--;
        }
        s->queue.clear();
        s->cv.notify_all();
    }
    if (s->thread.joinable()) s->thread.join();
    lf_ctx* c = s->ctx;
    std::lock_guard<std::recursive_mutex> g(c->mu);
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (auto& kv : s->jobs)
    {
        ServerJob& j = kv.second;
        for (auto& sp : j.inflight) cudaFreeAsync(sp.desc.radiance, c->stream);
        if (j.accum) cudaFreeAsync(j.accum, c->stream);
        if (j.doneEvent) cudaEventDestroy(j.doneEvent);
        if (j.engineJob >= 0) engine_job_free(s->engine, j.engineJob);
    }
    for (auto& kv : s->scenes)
        if (kv.second.dev) lf_scene_release(kv.second.dev);
    cudaStreamSynchronize(c->stream);
    delete s;
    return LF_OK;
}
}
