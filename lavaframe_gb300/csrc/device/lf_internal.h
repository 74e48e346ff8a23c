// Internal state of the C-ABI runtime objects, shared by the runtime (lf_runtime.cu), the
// multi-job engine driver (lf_engine_host.cu) and the serving loop (lf_server.cu).
#pragma once

#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "../../../include/lavaframe_gb300.h"
#include "lf_kernels.h"

using namespace lfd;

#include "lf_guide.cuh"

namespace lfrt
{
struct EngineHost;
void engine_destroy(EngineHost* e);
lfd::guide::Net guide_net(const lf_guide* g);
int guide_tensor_path(const lf_guide* g);
}

struct lf_ctx
{
    int device = 0;
    cudaStream_t stream = nullptr;
    std::recursive_mutex mu;
    std::string err;
    uint32_t* d_status = nullptr;
    unsigned long long* d_stats = nullptr;   // [3] traversal counters
    uint32_t devErrors = 0;
    uint64_t lastStats[3] = {0, 0, 0};
    // reusable device buffers of the host-pointer ray queries
    void* scratchRays = nullptr;
    size_t scratchRaysBytes = 0;
    void* scratchOut = nullptr;
    size_t scratchOutBytes = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    // pieces of the host-pointer ray queries: copy streams and one event per piece and side
    static constexpr int kMaxHostChunks = 8;
    int hostChunks = 0;                       // 0: automatic
    cudaStream_t copyIn = nullptr, copyOut = nullptr;
    cudaEvent_t chunkIn[kMaxHostChunks] = {}, chunkDone[kMaxHostChunks] = {};
    cudaEvent_t chunkStart = nullptr, chunkEnd = nullptr;
    // page-locked blocks from lf_host_alloc and their device addresses: results of host queries
    // whose output lies in one are written there by the kernels, without a copy back
    struct HostBlock
    {
        char* host;
        char* dev;
        size_t bytes;
    };
    std::vector<HostBlock> hostBlocks;
    // scratch of the binned ray queries
    uint32_t* binKeys = nullptr;
    int* binPerm = nullptr;
    size_t binCap = 0;
    uint32_t* binHist = nullptr;
    unsigned long long* binNext = nullptr;
    lfrt::EngineHost* engine = nullptr;   // multi-job engine, created on first use
    // traversal-kernel timer of the binned ray queries: one event pair per launch while on
    bool kernelTimer = false;
    std::vector<cudaEvent_t> ktEvents;     // start, stop, start, stop, ...
    size_t ktUsed = 0;                     // pairs recorded since the last read
};

struct lf_scene
{
    lf_ctx* ctx = nullptr;
    std::vector<void*> allocs;
    size_t bytes = 0;
    ShadeScene view{};
    // re-encoding metadata for instance updates
    int numRefNodes = 0;
    int topLevelIndex = 0;
    int numMeshNodes = 0;       // device records that belong to mesh levels
    std::vector<int> blasRootCode;   // per reference node index of a mesh root (code), lazily
    float4* d_nodes = nullptr;
    size_t nodeCapacity = 0;    // records allocated
    float4* d_instances = nullptr;
    ShadeInstance* d_sinst = nullptr;
    DevMaterial* d_materials = nullptr;
    int numMaterials = 0;
    std::vector<int> meshNodeMap;   // reference index -> device record (mesh levels), -1 otherwise
    float4* d_wide = nullptr;       // wide tree
    size_t wideCapacity = 0;        // wide records allocated
    float* d_refNodes = nullptr;    // the reference nodes (tie resolution)
    int* d_parent = nullptr;
    int* d_leafOfTri = nullptr;     // reference leaf of every triangle
    int* d_leafOfInst = nullptr;    // reference leaf of every instance
    float boundsLo[3] = {0, 0, 0}, boundsHi[3] = {0, 0, 0};   // instance-level root box
};

struct lf_frame
{
    lf_ctx* ctx = nullptr;
    lf_scene* scene = nullptr;
    Params P{};
    uint32_t flags = 0;
    int W = 0, H = 0;
    int numTilesX = 1, numTilesY = 1;
    int sppBatch = 0;
    long long cap = 0;   // path slots
    float4* accum = nullptr;
    double* accum64 = nullptr;
    PathSoA ps{};
    BounceBuffers bb{};
    std::vector<void*> fixedAllocs;   // accumulation buffers and counters
    std::vector<void*> allocs;        // path state and queues (sized by the batch)
    uint64_t paths = 0;
    int lastBatchSamples = 0;
    cudaGraphExec_t graph = nullptr;
    int graphDepth = -1;
    // engine path (default): job slot in the context's engine and the per-path radiance of
    // the most recent pass ([sample][pixel] of a single-tile frame)
    int engineJob = -1;
    float4* lastRadiance = nullptr;
    int lastRadianceSamples = 0;
    // learned path guiding (per-batch pipeline, one sample per batch)
    lf_guide* guide = nullptr;
    float guideAlpha = 0.5f;
    int guideTrainEvery = 4;
    float guideLr = 1e-2f;
    int guideTrainCap = 1 << 20;
    int guideBatch = 16384;        // samples per Adam step
    long long guideCap = 0;        // path slots the guide buffers hold
    GuideBuffers gb{};
    std::vector<void*> guideAllocs;
    uint64_t guideSteps = 0;
    uint64_t guideSamples = 0;
    uint64_t guideBatches = 0;     // guided batches rendered (training cadence)
};

namespace lfrt
{
inline lf_status fail(lf_ctx* c, lf_status st, const std::string& msg)
{
    if (c) c->err = msg;
    return st;
}

inline lf_status cuda_fail(lf_ctx* c, cudaError_t e, const char* what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return fail(c, LF_ERR_OOM, m);
    return fail(c, LF_ERR_CUDA, m);
}

template <class T>
inline cudaError_t dalloc(std::vector<void*>& list, size_t& bytes, T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
    if (e == cudaSuccess)
    {
        list.push_back(*p);
        bytes += sizeof(T) * count;
    }
    return e;
}

inline lf_status check_device(lf_ctx* c)
{
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "stream synchronize");
    uint32_t bits = 0;
    e = cudaMemcpy(&bits, c->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "status readback");
    if (bits)
    {
        c->devErrors |= bits;
        cudaMemset(c->d_status, 0, sizeof(uint32_t));
        return fail(c, LF_ERR_DEVICE, "device error bits 0x" + std::to_string(bits));
    }
    return LF_OK;
}

// Kernel parameters of one render (lf_render_params + scene facts); tile fields cover the
// whole frame unless the parameters set a tile size.
void fill_params(Params& P, const lf_render_params* p, const lf_scene* sc);

struct RefNode
{
    float bmin[3], bmax[3], lr[3];
};

inline float ulp_of(float x)
{
    x = std::fabs(x);
    float n = std::nextafter(x, INFINITY);
    return n - x;
}
}
