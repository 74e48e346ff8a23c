// Host-side state of the multi-job engine (implemented in lf_engine_host.cu).
#pragma once

#include "lf_engine.h"
#include "lf_internal.h"

namespace lfrt
{
struct EngineHost
{
    lf_ctx* c = nullptr;
    EngineBuffers b{};
    std::vector<void*> allocs;   // path pool and queues
    std::vector<void*> tables;   // job / pass tables, control block, counters
    size_t poolBytes = 0;
    unsigned long long* ownCtr = nullptr;   // counters of runs not tied to a frame
    EngineJob* h_jobStage = nullptr;        // pinned staging of the job table
    EnginePass* h_passStage = nullptr;      // pinned staging of the pass ring
    EngineCtl* h_ctl[2] = {nullptr, nullptr};
    unsigned long long* h_passDone[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    std::vector<char> jobUsed;
    unsigned long long total = 0;       // path ids handed out to passes
    unsigned long long numPasses = 0;   // passes submitted
    long long active = 0;               // passes submitted and not yet retired by their owner
    std::vector<unsigned> jobGen;       // bumped when a job's contents change
    struct Graph                        // two engine steps, captured per (counters, job)
    {
        cudaGraphExec_t exec = nullptr;
        unsigned long long* ctr = nullptr;
        int job = -1;                   // single job baked into the kernels, -1 = job table
        unsigned gen = 0;
        bool drain = false;             // drain form (launch_engine_drain)
    };
    std::vector<Graph> graphs;
    long long drainPaths = 1 << 22;     // paths left at which a frame run switches to the drain form (0 = never)
    int sortMode = 2;                   // sort-by-material: 0 off, 1 on, 2 single-job steps of mixed-class scenes
};

// Engine of the context, created on first use with the default pool size.
lf_status engine_get(lf_ctx* c, EngineHost** out);
// Pool slots (0 keeps the current pool), block sizes of extend / shade / shadow (0 = default)
// and the register cap of shade (threads per SM it must fit: 0 none, 512, 768, 1024).
lf_status engine_configure(EngineHost* e, int slots, int blockExtend, int blockShade, int blockShadow,
                           int shadeThreadsPerSm);
// Sort-by-material: extend buckets the hits by material class (4 x slots queue entries,
// allocated on first use) and shade takes them class by class. mode 0 off, 1 on, 2 (default)
// on for single-job steps whose scene has instances of more than one material class.
lf_status engine_set_sort(EngineHost* e, int mode);
int engine_job_alloc(EngineHost* e, const ShadeScene& S, const Params& P);
void engine_job_write(EngineHost* e, int job, const ShadeScene& S, const Params& P);
void engine_job_free(EngineHost* e, int job);
// Queues a pass descriptor (pathBase is assigned here); visible to the device after publish.
unsigned long long engine_pass_submit(EngineHost* e, EnginePass desc);
lf_status engine_publish(EngineHost* e);
// Enqueues one graph launch (two steps) counting into `ctr` (nullptr: the engine's own).
// job >= 0: every queued path belongs to that job (single-job kernels).
lf_status engine_launch_pair(EngineHost* e, unsigned long long* ctr, int job, bool drain = false);
// Enqueues a copy of the control block and pass counters into host buffer k and records ev[k].
lf_status engine_snapshot(EngineHost* e, int k);
// Runs steps until every submitted path has been written out.
lf_status engine_drain(EngineHost* e, unsigned long long* ctr, int maxDepth, int job);
// lf_frame_render on the engine: one pass per tile and sample chunk, accumulated in order.
lf_status frame_render_engine(lf_frame* f, const Params& P, int firstSample, int count);
}
