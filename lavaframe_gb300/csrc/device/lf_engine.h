// Persistent multi-job wavefront engine: device-side tables and launch interface
// (kernels in lf_engine.cu, host driver in lf_engine_host.cu).
//
// A fixed pool of path slots runs paths of many render passes at once. A pass is a range of
// samples of one tile of one job; its paths get consecutive global ids, and a slot whose path
// finished immediately starts the next unissued id (path regeneration), so the extension and
// shadow queues stay full until the work runs out instead of shrinking bounce by bounce.
// Each path writes its radiance into its pass's buffer ([sample][pixel of the visible tile])
// and the pass is accumulated per pixel in sample order once all its paths are done, so the
// image sums are the ones of the per-batch pipeline, bit for bit.
//
// One engine step with parity k (graph-captured, two steps per graph so the parity returns):
//   finish   done[k] (paths of depth-0 jobs): write them out, count pass completions, free
//            their slots
//   refill   start new paths in free slots while unissued ids remain (-> queue[k])
//   reset    commit the refill, clear done[k], the shadow queue and queue[k^1]
//   extend   closest hit of every queued path; hits and misses -> part (front and back), or
//            with sort-by-material the hits into one bucket per material class
//   shade    one PathTrace bounce over part's hits, then its misses, so that a warp shades
//            one kind; survivors -> queue[k^1]; a path that ends without next-event rays is
//            written out (radiance into its pass, completion counted, slot freed) on the spot
//   shadow   next-event visibility; writes out the paths that ended at the record's vertex
//   (the drain kernel writes out each path it runs to its end)
#pragma once

#include "lf_kernels.h"

namespace lfd
{
constexpr int kPassRingBits = 14;
constexpr int kPassRing = 1 << kPassRingBits;   // pass descriptors in flight
constexpr int kMaxEngineJobs = 1 << 16;         // job slots (packed into the upper bits of info.w)

struct EngineJob
{
    ShadeScene S;   // environment multiplier already applied
    Params P;       // job-level parameters; tile fields describe the tile size only
};

struct EnginePass
{
    int job;                     // job slot
    int firstSample, nSamples;
    int tileX, tileY, tileOrdinal;
    int visW, visH;              // visible part of the tile
    unsigned long long pathBase; // global id of the first path
    unsigned long long numPaths; // nSamples * visW * visH
    float4* radiance;            // numPaths entries, [sample][visible pixel]
};

struct EngineCtl
{
    unsigned long long next;       // next global path id to issue
    unsigned long long total;      // ids available
    unsigned long long passLo;     // first pass that may still have unissued ids
    unsigned long long numPasses;  // passes submitted
    int count[2];                  // extension queue sizes
    int shadowCount;
    int doneCount[2];              // done-list sizes
    int active;                    // paths started and not yet written out
    int freeCount;                 // free slots (info.w == -1)
    int taken;                     // slots the current step's refill started
    int extendNext, shadeNext, shadowNext;   // work counters of the extend, shade and shadow kernels
    int refillNext;                // ids handed out by the current refill
    int hitCount, missCount;       // the extension queue split by extend: hits, then misses
    int bucketCount[4];            // sort-by-material: hits per material class
};

struct EngineBuffers
{
    PathSoA ps;                  // info: x radiance entry in the pass, y depth, z last material, w ring | job << 14
    int* queue[2];
    int* part;                   // extended paths: hits from the front, misses from the back
    int* partSort;               // sort-by-material: hits of class k at [k * cap, k * cap + bucketCount[k])
    int sortByMaterial;          // 1: extend buckets hits by material class, shade takes them class by class
    ShadowRec* shadow;
    int* done[2];                // slots of depth-0 paths, written out by the next finish
    EngineCtl* ctl;
    const EngineJob* jobs;
    const EnginePass* passes;    // ring of kPassRing
    unsigned long long* passDone;// completed paths per ring entry
    uint32_t* status;
    unsigned long long* ctr;     // [1] extension rays, [2] shadow rays, [3] light-index clamps
    int cap;                     // pool slots
    int blockExtend, blockShade, blockShadow;
    int shadeThreadsPerSm;       // register cap of the shade kernel: 0 none, 512, 768 or 1024
};

// Launches one engine step with queue parity `parity` on `st`. With `one` set, every path
// belongs to that job and the kernels read it from their parameters (constant bank) instead
// of the job table.
int launch_engine_step(const EngineBuffers& b, const EngineJob* one, int parity, cudaStream_t st);
// Drain form of a step pair, for runs with few paths left: two steps whose extend / shade /
// shadow kernels are replaced by one kernel that runs every queued path to its end (one thread
// per path) and queues it as done. Leaves the parity where a step pair leaves it.
int launch_engine_drain(const EngineBuffers& b, const EngineJob* one, cudaStream_t st);
// Pool start: every slot on the done list, marked unused.
int launch_engine_init(const EngineBuffers& b, cudaStream_t st);
// Publishes newly written pass descriptors: clamps the overshoot of `next` to the old total,
// then raises total / numPasses and advances passLo past fully issued passes.
int launch_engine_append(const EngineBuffers& b, unsigned long long total, unsigned long long numPasses,
                         cudaStream_t st);
// Per-pixel in-order sum of one completed pass into the job's accumulation buffers.
int launch_engine_accumulate(const Params& P, const EnginePass& pass, float4* accum, double* accum64,
                             cudaStream_t st);
}
