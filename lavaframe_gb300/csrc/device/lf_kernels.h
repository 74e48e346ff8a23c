// Launch interface of the wavefront kernels and ray queries (implemented in lf_kernels.cu).
#pragma once

#include "lf_guide.cuh"
#include "lf_shade.cuh"

namespace lfd
{
// Per-path state, structure of arrays, one slot per (sample, pixel) of a batch.
struct PathSoA
{
    float4* o;      // ray origin, w = pdf of the last BSDF sample (MIS at the next hit)
    float4* d;      // ray direction
    float4* T;      // throughput
    float4* L;      // radiance
    float4* A;      // absorption coefficient
    uint4* rng;     // PCG4D state
    int4* info;     // x: pixel index (-1 = off screen), y: depth, z: last material
    float2* luv;    // texture coordinate of the last triangle hit
    float4* hit;    // t, instance, packed triangle, light (int bits)
};

// Next-event rays of one path: up to an environment ray and a light ray plus their
// unoccluded contributions and the throughput they are weighted by.
struct ShadowRec
{
    float4 a;   // surface position, w: path slot (int bits)
    float4 b;   // throughput, w: flags (1 env ray, 2 light ray; engine: 4 the path ends after these rays)
    float4 c;   // environment direction
    float4 e;   // environment contribution
    float4 f;   // light direction, w: max distance
    float4 g;   // light contribution
};

struct BounceBuffers
{
    int* queue[2];
    int* count;          // [2] queue sizes
    ShadowRec* shadow;
    int* shadowCount;
    uint32_t* status;
    unsigned long long* ctr;   // [0] paths, [1] extension rays, [2] shadow rays, [3] light clamps
    unsigned long long* fetch; // [2] work counters of the extend / shadow kernels
};

// Floats per recorded path vertex of guided rendering (see GuideCtx in lf_pathops.cuh).
constexpr int kGuideRecFloats = 20;

// Guided bounces (learned path guiding): per-queue-position queries and mixtures, per-slot
// training records, and the training sample buffer of the batch.
struct GuideBuffers
{
    guide::Net net;
    float* queries;      // cap x guide::kSampleFloats
    float* mix;          // cap x guide::kMixFloats
    float* rec;          // maxDepth x 20 fields x the batch's path slots, or null when the batch is not recorded
    float* train;        // trainCap x guide::kSampleFloats
    int* trainCount;
    int trainCap;
    float alpha;         // mixture selection probability
    int maxDepth;
    float weightClamp;   // training weights are clamped to this
    int tensorPath;      // 1: MLP inference on tcgen05 (lf_guide_tc.cu), 0: warp-level mma.sync
};

int launch_bounce_guided(const ShadeScene& S, const Params& P, const PathSoA& ps, const BounceBuffers& b,
                         const GuideBuffers& g, int bounce, long long cap, cudaStream_t st);
// Training samples from the recorded vertices of the batch's n paths.
int launch_guide_collect(const PathSoA& ps, const GuideBuffers& g, long long n, cudaStream_t st);

// Resident blocks per SM of `kernel` at `block` threads (the occupancy query, remembered per
// kernel and block size: the query costs more host time than a launch).
int occupancy_blocks_per_sm(const void* kernel, int block, size_t dynamicSmem = 0);

int launch_generate(const ShadeScene& S, const Params& P, const PathSoA& ps, int firstSample, int nSamples,
                    int* queue, int* qcount, cudaStream_t st);
int launch_bounce(const ShadeScene& S, const Params& P, const PathSoA& ps, const BounceBuffers& b, int bounce,
                  long long cap, cudaStream_t st);
int launch_accumulate(const Params& P, const PathSoA& ps, int nSamples, float4* accum, double* accum64,
                      cudaStream_t st);
int launch_trace_closest(const DevScene& S, const float4* rays, long long n, int4* hits, int lights, bool stats,
                         uint32_t* status, unsigned long long* stat3, cudaStream_t st);
// evStart / evStop (optional) are recorded on `st` around the traversal kernel alone.
int launch_trace_binned(const DevScene& S, const float4* rays, long long n, void* out, bool any, int lights,
                        const float lo[3], const float hi[3], bool binning, uint32_t* keys, uint32_t* hist, int* perm,
                        unsigned long long* next, uint32_t* status, cudaStream_t st, cudaEvent_t evStart = nullptr,
                        cudaEvent_t evStop = nullptr);
int trace_bins();
int launch_trace_any(const DevScene& S, const float4* rays, long long n, uint8_t* occ, int lights, bool stats,
                     uint32_t* status, unsigned long long* stat3, cudaStream_t st);
}
