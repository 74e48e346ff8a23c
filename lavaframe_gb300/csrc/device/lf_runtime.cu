// C-ABI runtime: device context, scene upload (re-encoding of the reference flat arrays
// into the traversal layout described in lf_device.cuh), ray queries and progressive
// render targets. Host code here must be compiled with -ffp-contract=off: light
// precomputation and matrix inverses are part of the arithmetic contract.
#include <algorithm>
#include <limits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "lf_engine_host.h"
#include "lf_pixel.h"

using namespace lfrt;

extern "C" {

lf_status lf_ctx_create(int32_t device, lf_ctx** out)
{
    if (!out) return LF_ERR_INVALID;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return LF_ERR_CUDA;
    if (device < 0 || device >= count) return LF_ERR_INVALID;
    lf_ctx* c = new lf_ctx;
    c->device = device;
    if ((e = cudaSetDevice(device)) != cudaSuccess || (e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaMalloc((void**)&c->d_status, sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaMalloc((void**)&c->d_stats, 3 * sizeof(unsigned long long))) != cudaSuccess)
    {
        delete c;
        return e == cudaErrorMemoryAllocation ? LF_ERR_OOM : LF_ERR_CUDA;
    }
    cudaMemset(c->d_status, 0, sizeof(uint32_t));
    cudaMemset(c->d_stats, 0, 3 * sizeof(unsigned long long));
    *out = c;
    return LF_OK;
}

void lf_ctx_destroy(lf_ctx* c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    engine_destroy(c->engine);
    c->engine = nullptr;
    cudaFree(c->d_status);
    cudaFree(c->d_stats);
    cudaFree(c->scratchRays);
    cudaFree(c->scratchOut);
    cudaFree(c->binKeys);
    cudaFree(c->binPerm);
    cudaFree(c->binHist);
    cudaFree(c->binNext);
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
    for (int k = 0; k < lf_ctx::kMaxHostChunks; ++k)
    {
        if (c->chunkIn[k]) cudaEventDestroy(c->chunkIn[k]);
        if (c->chunkDone[k]) cudaEventDestroy(c->chunkDone[k]);
    }
    for (cudaEvent_t ev : c->ktEvents) cudaEventDestroy(ev);
    if (c->chunkStart) cudaEventDestroy(c->chunkStart);
    if (c->chunkEnd) cudaEventDestroy(c->chunkEnd);
    if (c->copyIn) cudaStreamDestroy(c->copyIn);
    if (c->copyOut) cudaStreamDestroy(c->copyOut);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char* lf_ctx_last_error(const lf_ctx* c) { return c ? c->err.c_str() : "null context"; }
uint32_t lf_ctx_device_errors(const lf_ctx* c) { return c ? c->devErrors : 0; }

lf_status lf_ctx_sync(lf_ctx* c)
{
    if (!c) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    return check_device(c);
}

lf_status lf_ctx_timer_start(lf_ctx* c)
{
    if (!c) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    for (auto& e : c->ev)
        if (!e && cudaEventCreate(&e) != cudaSuccess) return fail(c, LF_ERR_CUDA, "event create");
    cudaError_t e = cudaEventRecord(c->ev[0], c->stream);
    return e == cudaSuccess ? LF_OK : cuda_fail(c, e, "event record");
}

lf_status lf_ctx_timer_stop(lf_ctx* c, float* ms)
{
    if (!c || !ms || !c->ev[0]) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    cudaError_t e = cudaEventRecord(c->ev[1], c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(c->ev[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, c->ev[0], c->ev[1]);
    return e == cudaSuccess ? LF_OK : cuda_fail(c, e, "event timing");
}

lf_status lf_ctx_device_attrs(lf_ctx* c, int32_t* sm_count, int32_t* max_sm_mhz)
{
    if (!c || !sm_count || !max_sm_mhz) return LF_ERR_INVALID;
    int sms = 0, khz = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, c->device);
    if (e != cudaSuccess) return cuda_fail(c, e, "device attributes");
    *sm_count = sms;
    *max_sm_mhz = khz / 1000;
    return LF_OK;
}

lf_status lf_ctx_kernel_timer(lf_ctx* c, int32_t on)
{
    if (!c) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    c->kernelTimer = on != 0;
    c->ktUsed = 0;
    return LF_OK;
}

lf_status lf_ctx_kernel_timer_read(lf_ctx* c, double* total_ms, int64_t* launches)
{
    if (!c || !total_ms || !launches) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    double sum = 0.0;
    for (size_t k = 0; k < c->ktUsed; ++k)
    {
        cudaError_t e = cudaEventSynchronize(c->ktEvents[2 * k + 1]);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, c->ktEvents[2 * k], c->ktEvents[2 * k + 1]);
        if (e != cudaSuccess) return cuda_fail(c, e, "kernel timer");
        sum += ms;
    }
    *total_ms = sum;
    *launches = (int64_t)c->ktUsed;
    c->ktUsed = 0;
    return LF_OK;
}

lf_status lf_host_alloc(lf_ctx* c, size_t bytes, void** out)
{
    if (!c || !out) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    const size_t size = bytes ? bytes : 1;
    cudaError_t e = cudaHostAlloc(out, size, cudaHostAllocMapped);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaHostAlloc");
    void* dev = nullptr;
    if (cudaHostGetDevicePointer(&dev, *out, 0) != cudaSuccess)
    {
        cudaGetLastError();
        dev = nullptr;   // not reachable from kernels: host queries copy their results back
    }
    c->hostBlocks.push_back({(char*)*out, (char*)dev, size});
    return LF_OK;
}

lf_status lf_host_free(lf_ctx* c, void* p)
{
    if (!c) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    for (size_t i = 0; i < c->hostBlocks.size(); ++i)
        if (c->hostBlocks[i].host == (char*)p)
        {
            c->hostBlocks.erase(c->hostBlocks.begin() + (long)i);
            break;
        }
    cudaError_t e = cudaFreeHost(p);
    return e == cudaSuccess ? LF_OK : cuda_fail(c, e, "cudaFreeHost");
}

lf_status lf_device_alloc(lf_ctx* c, size_t bytes, void** out)
{
    if (!c || !out) return LF_ERR_INVALID;
    cudaSetDevice(c->device);
    cudaError_t e = cudaMalloc(out, bytes ? bytes : 1);
    return e == cudaSuccess ? LF_OK : cuda_fail(c, e, "cudaMalloc");
}

lf_status lf_device_free(lf_ctx* c, void* p)
{
    if (!c) return LF_ERR_INVALID;
    cudaSetDevice(c->device);
    cudaError_t e = cudaFree(p);
    return e == cudaSuccess ? LF_OK : cuda_fail(c, e, "cudaFree");
}

lf_status lf_copy_to_device(lf_ctx* c, void* dst, const void* src, size_t bytes)
{
    if (!c) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? LF_OK : cuda_fail(c, e, "copy to device");
}

lf_status lf_copy_to_host(lf_ctx* c, void* dst, const void* src, size_t bytes)
{
    if (!c) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? LF_OK : cuda_fail(c, e, "copy to host");
}

// ------------------------------------------------------------------ scene upload
namespace
{
// Builds the device records for the instance level starting at the reference index
// `top`, appending to `recs`. Returns the root code.
lf_status encode_level(lf_ctx* c, const RefNode* nodes, int numNodes, int start, bool meshLevel, int numTris,
                       int numInstances, std::vector<float4>& recs, std::vector<int>& map, int* rootCode)
{
    auto leaf_code = [&](const RefNode& n, int* code) -> bool {
        int z = (int)n.lr[2];
        if (meshLevel)
        {
            if (z <= 0) return false;
            int first = (int)n.lr[0], cnt = (int)n.lr[1];
            if (first < 0 || cnt < 0 || cnt > 3 || first + cnt > numTris) return false;
            *code = ~((first << 2) | cnt);
        }
        else
        {
            if (z >= 0) return false;
            int inst = -z - 1;
            if (inst >= numInstances) return false;
            *code = ~inst;
        }
        return true;
    };
    if (start < 0 || start >= numNodes) return fail(c, LF_ERR_INVALID, "node index out of range");
    const RefNode& r = nodes[start];
    if ((int)r.lr[2] != 0)
    {
        if (!leaf_code(r, rootCode)) return fail(c, LF_ERR_INVALID, "bad leaf node " + std::to_string(start));
        return LF_OK;
    }
    if (map[start] >= 0)
    {
        *rootCode = map[start];
        return LF_OK;
    }
    // iterative pre-order: assign records parent-first
    struct Item { int ref; };
    std::vector<int> stack{start};
    map[start] = (int)(recs.size() / 4);
    recs.resize(recs.size() + 4);
    while (!stack.empty())
    {
        int ref = stack.back();
        stack.pop_back();
        const RefNode& n = nodes[ref];
        int rec = map[ref];
        int child[2] = {(int)n.lr[0], (int)n.lr[1]};
        int code[2];
        for (int k = 0; k < 2; ++k)
        {
            int ci = child[k];
            if (ci < 0 || ci >= numNodes) return fail(c, LF_ERR_INVALID, "child index out of range at node " + std::to_string(ref));
            const RefNode& cn = nodes[ci];
            if ((int)cn.lr[2] != 0)
            {
                if (!leaf_code(cn, &code[k])) return fail(c, LF_ERR_INVALID, "bad leaf node " + std::to_string(ci));
            }
            else
            {
                if (map[ci] >= 0) return fail(c, LF_ERR_INVALID, "node referenced twice: " + std::to_string(ci));
                map[ci] = (int)(recs.size() / 4);
                recs.resize(recs.size() + 4);
                code[k] = map[ci];
            }
        }
        const RefNode& L = nodes[child[0]];
        const RefNode& R = nodes[child[1]];
        float4* o = &recs[(size_t)rec * 4];
        o[0] = make_float4(L.bmin[0], L.bmin[1], L.bmin[2], L.bmax[0]);
        o[1] = make_float4(L.bmax[1], L.bmax[2], R.bmin[0], R.bmin[1]);
        o[2] = make_float4(R.bmin[2], R.bmax[0], R.bmax[1], R.bmax[2]);
        float cf0, cf1;
        std::memcpy(&cf0, &code[0], 4);
        std::memcpy(&cf1, &code[1], 4);
        o[3] = make_float4(cf0, cf1, 0.f, 0.f);
        // push right then left so the left subtree is laid out first
        if ((int)R.lr[2] == 0) stack.push_back(child[1]);
        if ((int)L.lr[2] == 0) stack.push_back(child[0]);
    }
    *rootCode = map[start];
    return LF_OK;
}

// ------------------------------------------------------------------ wide (4-way) tree
// Every wide node holds up to four reference nodes as children: starting from a reference
// inner node's two children, the inner child with the largest box surface area is replaced by
// its two children until four children are reached or only leaves remain. Leaves keep the
// binary encoding's codes; every child slot carries the reference node's own box and index.
struct WideBuilder
{
    const RefNode* nodes = nullptr;
    int numNodes = 0, numTris = 0, numInstances = 0;
    std::vector<float4> recs;
    std::vector<int> map;   // reference inner node -> wide record it heads
};

bool ref_leaf_code(const RefNode& n, bool meshLevel, int numTris, int numInstances, int* code)
{
    const int z = (int)n.lr[2];
    if (meshLevel)
    {
        if (z <= 0) return false;
        const int first = (int)n.lr[0], cnt = (int)n.lr[1];
        if (first < 0 || cnt < 0 || cnt > 3 || first + cnt > numTris) return false;
        *code = ~((first << 2) | cnt);
    }
    else
    {
        if (z >= 0) return false;
        const int inst = -z - 1;
        if (inst >= numInstances) return false;
        *code = ~inst;
    }
    return true;
}

float box_area(const RefNode& n)
{
    const float dx = n.bmax[0] - n.bmin[0], dy = n.bmax[1] - n.bmin[1], dz = n.bmax[2] - n.bmin[2];
    return dx * dy + dy * dz + dz * dx;
}

lf_status wide_level(lf_ctx* c, WideBuilder& B, int start, bool meshLevel, int* rootCode)
{
    if (start < 0 || start >= B.numNodes) return fail(c, LF_ERR_INVALID, "node index out of range");
    const RefNode& r = B.nodes[start];
    if ((int)r.lr[2] != 0)
    {
        if (!ref_leaf_code(r, meshLevel, B.numTris, B.numInstances, rootCode))
            return fail(c, LF_ERR_INVALID, "bad leaf node " + std::to_string(start));
        return LF_OK;
    }
    if (B.map[start] >= 0)
    {
        *rootCode = B.map[start];
        return LF_OK;
    }
    auto inner = [&](int i) { return (int)B.nodes[i].lr[2] == 0; };
    B.map[start] = (int)(B.recs.size() / kWideF4);
    B.recs.resize(B.recs.size() + kWideF4);
    std::vector<int> stack{start};
    while (!stack.empty())
    {
        const int ref = stack.back();
        stack.pop_back();
        const int rec = B.map[ref];
        std::vector<int> kids{(int)B.nodes[ref].lr[0], (int)B.nodes[ref].lr[1]};
        for (int k : kids)
            if (k < 0 || k >= B.numNodes) return fail(c, LF_ERR_INVALID, "child index out of range");
        while ((int)kids.size() < kWide)
        {
            int best = -1;
            float area = -1.f;
            for (int k = 0; k < (int)kids.size(); ++k)
                if (inner(kids[k]) && box_area(B.nodes[kids[k]]) > area)
                {
                    area = box_area(B.nodes[kids[k]]);
                    best = k;
                }
            if (best < 0) break;
            const int x = kids[best];
            const int xl = (int)B.nodes[x].lr[0], xr = (int)B.nodes[x].lr[1];
            if (xl < 0 || xl >= B.numNodes || xr < 0 || xr >= B.numNodes)
                return fail(c, LF_ERR_INVALID, "child index out of range");
            kids[best] = xl;
            kids.insert(kids.begin() + best + 1, xr);
        }
        float f[8][kWide];
        for (int j = 0; j < kWide; ++j)
        {
            int code = kWideEmpty, refIdx = -1;
            // an unused slot gets the empty box lo = +inf, hi = -inf: read in near / far order
            // (wide_slabs) its entry is +inf and its exit -inf for every ray, so no test passes
            const float inf = std::numeric_limits<float>::infinity();
            float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
            if (j < (int)kids.size())
            {
                const int k = kids[j];
                const RefNode& n = B.nodes[k];
                for (int a = 0; a < 3; ++a)
                {
                    lo[a] = n.bmin[a];
                    hi[a] = n.bmax[a];
                }
                refIdx = k;
                if (inner(k))
                {
                    if (B.map[k] >= 0) return fail(c, LF_ERR_INVALID, "node referenced twice: " + std::to_string(k));
                    B.map[k] = (int)(B.recs.size() / kWideF4);
                    B.recs.resize(B.recs.size() + kWideF4);
                    code = B.map[k];
                    stack.push_back(k);
                }
                else if (!ref_leaf_code(n, meshLevel, B.numTris, B.numInstances, &code))
                    return fail(c, LF_ERR_INVALID, "bad leaf node " + std::to_string(k));
            }
            f[0][j] = lo[0];
            f[1][j] = hi[0];
            f[2][j] = lo[1];
            f[3][j] = hi[1];
            f[4][j] = lo[2];
            f[5][j] = hi[2];
            std::memcpy(&f[6][j], &code, 4);
            std::memcpy(&f[7][j], &refIdx, 4);
        }
        float4* o = &B.recs[(size_t)rec * kWideF4];
        for (int g = 0; g < 8; ++g)
            for (int h4 = 0; h4 < kWide / 4; ++h4)
                o[g * (kWide / 4) + h4] = make_float4(f[g][h4 * 4], f[g][h4 * 4 + 1], f[g][h4 * 4 + 2], f[g][h4 * 4 + 3]);
    }
    *rootCode = B.map[start];
    return LF_OK;
}

// Wide tree of the whole scene (mesh levels first, then the instance level), the instance
// records' wide root codes and mesh root reference nodes, the reference parent array and the
// reference leaf that holds each triangle and each instance (tie resolution only).
lf_status encode_wide(lf_ctx* c, const lf_scene_view* v, const RefNode* nodes, std::vector<float4>& inst,
                      std::vector<float4>& wrecs, std::vector<int>& parent, std::vector<int>& leafOfTri,
                      std::vector<int>& leafOfInst, int* wroot)
{
    WideBuilder B;
    B.nodes = nodes;
    B.numNodes = v->num_nodes;
    B.numTris = v->num_tris;
    B.numInstances = v->num_instances;
    B.map.assign(v->num_nodes, -1);
    std::vector<int> instRoot(v->num_instances, -1);
    std::vector<int> stack{v->top_level_index};
    while (!stack.empty())
    {
        const int ref = stack.back();
        stack.pop_back();
        const RefNode& n = nodes[ref];
        const int z = (int)n.lr[2];
        if (z < 0)
            instRoot[-z - 1] = (int)n.lr[0];
        else if (z == 0)
        {
            stack.push_back((int)n.lr[1]);
            stack.push_back((int)n.lr[0]);
        }
    }
    for (int i = 0; i < v->num_instances; ++i)
    {
        int code = ~0, rootRef = -1;
        if (instRoot[i] >= 0)
        {
            lf_status st = wide_level(c, B, instRoot[i], true, &code);
            if (st != LF_OK) return st;
            rootRef = instRoot[i];
        }
        float cf, rf;
        std::memcpy(&cf, &code, 4);
        std::memcpy(&rf, &rootRef, 4);
        inst[(size_t)i * 4 + 3].z = cf;
        inst[(size_t)i * 4 + 3].w = rf;
    }
    lf_status st = wide_level(c, B, v->top_level_index, false, wroot);
    if (st != LF_OK) return st;
    wrecs.swap(B.recs);
    parent.assign(v->num_nodes, -1);
    leafOfTri.assign(std::max(v->num_tris, 1), -1);
    leafOfInst.assign(std::max(v->num_instances, 1), -1);
    for (int i = 0; i < v->num_nodes; ++i)
    {
        const int z = (int)nodes[i].lr[2];
        const int l = (int)nodes[i].lr[0], r = (int)nodes[i].lr[1];
        if (z == 0)
        {
            if (l >= 0 && l < v->num_nodes) parent[l] = i;
            if (r >= 0 && r < v->num_nodes) parent[r] = i;
        }
        else if (z > 0)
        {
            for (int t = std::max(l, 0); t < l + r && t < v->num_tris; ++t) leafOfTri[t] = i;
        }
        else if (-z - 1 < v->num_instances)
            leafOfInst[-z - 1] = i;
    }
    return LF_OK;
}

void make_light(const float* l15, DevLight& d)
{
    using lfc::v3;
    std::memset(&d, 0, sizeof d);
    for (int k = 0; k < 3; ++k)
    {
        d.pos[k] = l15[k];
        d.emission[k] = l15[3 + k];
        d.u[k] = l15[6 + k];
        d.v[k] = l15[9 + k];
    }
    d.radius = l15[12];
    d.area = l15[13];
    d.type = l15[14];
    v3 u(d.u[0], d.u[1], d.u[2]), v(d.v[0], d.v[1], d.v[2]), p(d.pos[0], d.pos[1], d.pos[2]);
    v3 n = lfc::normalize(lfc::cross(u, v));
    d.normal[0] = n.x; d.normal[1] = n.y; d.normal[2] = n.z;
    d.planeW = lfc::dot(n, p);
    v3 us = u * (1.0f / lfc::dot(u, u));
    v3 vs = v * (1.0f / lfc::dot(v, v));
    d.us[0] = us.x; d.us[1] = us.y; d.us[2] = us.z;
    d.vs[0] = vs.x; d.vs[1] = vs.y; d.vs[2] = vs.z;
}

// Instance-level root box (the ray-binning grid of the batched queries).
void set_bounds(lf_scene* sc, const RefNode& root)
{
    for (int k = 0; k < 3; ++k)
    {
        sc->boundsLo[k] = root.bmin[k];
        sc->boundsHi[k] = root.bmax[k];
    }
}

uint32_t shade_class_mask(const std::vector<ShadeInstance>& sinst)
{
    uint32_t m = 0;
    for (const ShadeInstance& s : sinst) m |= 1u << (s.shadeClass & 3);
    return m;
}

lf_status encode_instances(lf_ctx* c, const lf_scene_view* v, const RefNode* nodes, std::vector<float4>& recs,
                           std::vector<int>& map, std::vector<float4>& inst, std::vector<ShadeInstance>& sinst,
                           int* tlasRoot)
{
    const int ni = v->num_instances;
    // instance level
    lf_status st = encode_level(c, nodes, v->num_nodes, v->top_level_index, false, v->num_tris, ni, recs, map, tlasRoot);
    if (st != LF_OK) return st;
    // instance records from the instance-level leaves
    std::vector<int> instRootRef(ni, -1), instMat(ni, -1);
    std::vector<int> stack{v->top_level_index};
    while (!stack.empty())
    {
        int ref = stack.back();
        stack.pop_back();
        const RefNode& n = nodes[ref];
        int z = (int)n.lr[2];
        if (z < 0)
        {
            int i = -z - 1;
            if (instRootRef[i] != -1) return fail(c, LF_ERR_INVALID, "instance listed twice in the instance tree");
            instRootRef[i] = (int)n.lr[0];
            instMat[i] = (int)n.lr[1];
        }
        else if (z == 0)
        {
            stack.push_back((int)n.lr[1]);
            stack.push_back((int)n.lr[0]);
        }
        else
            return fail(c, LF_ERR_INVALID, "mesh leaf inside the instance tree");
    }
    inst.assign((size_t)ni * 4, make_float4(0, 0, 0, 0));
    sinst.assign(ni, ShadeInstance{});
    for (int i = 0; i < ni; ++i)
    {
        const float* M = v->transforms + (size_t)i * 16;
        float inv[16];
        lfc::inverse4(M, inv);
        int rootCode = ~0;   // empty leaf for instances that no leaf references
        if (instRootRef[i] >= 0)
        {
            st = encode_level(c, nodes, v->num_nodes, instRootRef[i], true, v->num_tris, ni, recs, map, &rootCode);
            if (st != LF_OK) return st;
            if (instMat[i] < 0 || instMat[i] >= v->num_materials)
                return fail(c, LF_ERR_INVALID, "instance material out of range");
        }
        float rc, mc;
        int mat = instMat[i] < 0 ? 0 : instMat[i];
        std::memcpy(&rc, &rootCode, 4);
        std::memcpy(&mc, &mat, 4);
        float4* o = &inst[(size_t)i * 4];
        // columns c0..c3 (xyz) of the inverse
        o[0] = make_float4(inv[0], inv[1], inv[2], inv[4]);
        o[1] = make_float4(inv[5], inv[6], inv[8], inv[9]);
        o[2] = make_float4(inv[10], inv[12], inv[13], inv[14]);
        o[3] = make_float4(rc, mc, 0.f, 0.f);
        ShadeInstance& s = sinst[i];
        for (int col = 0; col < 4; ++col)
            for (int r = 0; r < 3; ++r) s.fwd[col * 3 + r] = M[col * 4 + r];
        lfc::normal_matrix(M, s.nrm);
        s.material = mat;
        // class of the material's shading code (Material.h layout: metallic [8], transmission
        // [16], texture ids [24..27]) for the engine's sort-by-material
        const float* mp = v->materials + (size_t)mat * 28;
        const bool textured = mp[24] >= 0.f || mp[25] >= 0.f || mp[26] >= 0.f || mp[27] >= 0.f;
        s.shadeClass = textured ? 3 : mp[16] > 0.f ? 2 : mp[8] >= 0.5f ? 1 : 0;
    }
    return LF_OK;
}
}

lf_status lf_scene_upload(lf_ctx* c, const lf_scene_view* v, lf_scene** out)
{
    if (!c || !v || !out) return LF_ERR_INVALID;
    *out = nullptr;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    if (v->num_nodes <= 0 || !v->nodes || v->num_tris <= 0 || !v->vert_indices || v->num_vertices <= 0 ||
        !v->vertices_uvx || !v->normals_uvy || v->num_materials <= 0 || !v->materials || v->num_instances <= 0 ||
        !v->transforms || v->top_level_index < 0 || v->top_level_index >= v->num_nodes ||
        (v->num_lights > 0 && !v->lights))
        return fail(c, LF_ERR_INVALID, "incomplete scene view");
    const RefNode* nodes = reinterpret_cast<const RefNode*>(v->nodes);

    std::vector<float4> recs;
    recs.reserve((size_t)v->num_nodes * 4);
    std::vector<int> map(v->num_nodes, -1);
    std::vector<float4> inst;
    std::vector<ShadeInstance> sinst;
    int tlasRoot = 0;
    lf_status st = encode_instances(c, v, nodes, recs, map, inst, sinst, &tlasRoot);
    if (st != LF_OK) return st;
    std::vector<float4> wrecs;
    std::vector<int> parent, leafOfTri, leafOfInst;
    int wroot = 0;
    st = encode_wide(c, v, nodes, inst, wrecs, parent, leafOfTri, leafOfInst, &wroot);
    if (st != LF_OK) return st;
    // room for a re-encoded instance level after instance updates (at most one wide node per
    // inner node of the instance tree)
    const size_t wideCap = wrecs.size() / kWideF4 + (size_t)v->num_instances;

    // triangles in packed order: v0, v1 - v0, v2 - v0
    std::vector<float4> tris((size_t)v->num_tris * 3);
    std::vector<int4> vidx(v->num_tris);
    float extent = 0.f;
    for (int k = 0; k < v->num_tris; ++k)
    {
        const int* ix = v->vert_indices + (size_t)k * 3;
        for (int j = 0; j < 3; ++j)
            if (ix[j] < 0 || ix[j] >= v->num_vertices) return fail(c, LF_ERR_INVALID, "vertex index out of range");
        const float* a = v->vertices_uvx + (size_t)ix[0] * 4;
        const float* b = v->vertices_uvx + (size_t)ix[1] * 4;
        const float* cc = v->vertices_uvx + (size_t)ix[2] * 4;
        tris[(size_t)k * 3 + 0] = make_float4(a[0], a[1], a[2], 0.f);
        tris[(size_t)k * 3 + 1] = make_float4(b[0] - a[0], b[1] - a[1], b[2] - a[2], 0.f);
        tris[(size_t)k * 3 + 2] = make_float4(cc[0] - a[0], cc[1] - a[1], cc[2] - a[2], 0.f);
        vidx[k] = make_int4(ix[0], ix[1], ix[2], 0);
    }
    for (int i = 0; i < v->num_nodes; ++i)
        for (int k = 0; k < 3; ++k)
        {
            float m = std::max(std::fabs(nodes[i].bmin[k]), std::fabs(nodes[i].bmax[k]));
            if (m < 3.0e38f) extent = std::max(extent, m);
        }

    std::vector<DevLight> lights(std::max(v->num_lights, 0));
    for (int i = 0; i < v->num_lights; ++i) make_light(v->lights + (size_t)i * 15, lights[i]);

    lf_scene* sc = new lf_scene;
    sc->ctx = c;
    cudaError_t e = cudaSuccess;
    float4 *d_nodes, *d_tris, *d_inst, *d_verts, *d_norms;
    DevLight* d_lights;
    int4* d_vidx;
    DevMaterial* d_mats;
    ShadeInstance* d_sinst;
    auto A = [&](auto** p, size_t n) {
        if (e == cudaSuccess) e = dalloc(sc->allocs, sc->bytes, p, n);
    };
    A(&d_nodes, recs.size());
    A(&d_tris, tris.size());
    A(&d_inst, inst.size());
    A(&d_lights, lights.size());
    A(&d_vidx, vidx.size());
    A(&d_verts, (size_t)v->num_vertices);
    A(&d_norms, (size_t)v->num_vertices);
    A(&d_mats, (size_t)v->num_materials);
    A(&d_sinst, sinst.size());
    float4* d_wide = nullptr;
    float* d_refNodes = nullptr;
    int* d_parent = nullptr;
    int *d_leafOfTri = nullptr, *d_leafOfInst = nullptr;
    A(&d_wide, wideCap * kWideF4);
    A(&d_refNodes, (size_t)v->num_nodes * 9);
    A(&d_parent, (size_t)v->num_nodes);
    A(&d_leafOfTri, leafOfTri.size());
    A(&d_leafOfInst, leafOfInst.size());
    float* d_env = nullptr;
    float2 *d_marg = nullptr, *d_cond = nullptr;
    uint8_t* d_tex = nullptr;
    bool hasEnv = v->env_rgb && v->env_width > 0 && v->env_height > 0 && v->env_marginal && v->env_conditional;
    if (hasEnv)
    {
        A(&d_env, (size_t)v->env_width * v->env_height * 3);
        A(&d_marg, (size_t)v->env_height);
        A(&d_cond, (size_t)v->env_width * v->env_height);
    }
    bool hasTex = v->textures && v->num_textures > 0 && v->tex_width > 0 && v->tex_height > 0;
    if (hasTex) A(&d_tex, (size_t)v->num_textures * v->tex_width * v->tex_height * 4);
    if (e != cudaSuccess)
    {
        lf_scene_release(sc);
        return cuda_fail(c, e, "scene allocation");
    }
    auto H2D = [&](void* dst, const void* src, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    };
    H2D(d_nodes, recs.data(), recs.size() * sizeof(float4));
    H2D(d_tris, tris.data(), tris.size() * sizeof(float4));
    H2D(d_inst, inst.data(), inst.size() * sizeof(float4));
    H2D(d_lights, lights.data(), lights.size() * sizeof(DevLight));
    H2D(d_vidx, vidx.data(), vidx.size() * sizeof(int4));
    H2D(d_verts, v->vertices_uvx, (size_t)v->num_vertices * 16);
    H2D(d_norms, v->normals_uvy, (size_t)v->num_vertices * 16);
    H2D(d_mats, v->materials, (size_t)v->num_materials * sizeof(DevMaterial));
    H2D(d_sinst, sinst.data(), sinst.size() * sizeof(ShadeInstance));
    H2D(d_wide, wrecs.data(), wrecs.size() * sizeof(float4));
    H2D(d_refNodes, v->nodes, (size_t)v->num_nodes * 9 * sizeof(float));
    H2D(d_parent, parent.data(), parent.size() * sizeof(int));
    H2D(d_leafOfTri, leafOfTri.data(), leafOfTri.size() * sizeof(int));
    H2D(d_leafOfInst, leafOfInst.data(), leafOfInst.size() * sizeof(int));
    if (hasEnv)
    {
        H2D(d_env, v->env_rgb, (size_t)v->env_width * v->env_height * 3 * sizeof(float));
        H2D(d_marg, v->env_marginal, (size_t)v->env_height * sizeof(float2));
        H2D(d_cond, v->env_conditional, (size_t)v->env_width * v->env_height * sizeof(float2));
    }
    if (hasTex) H2D(d_tex, v->textures, (size_t)v->num_textures * v->tex_width * v->tex_height * 4);
    if (e != cudaSuccess)
    {
        lf_scene_release(sc);
        return cuda_fail(c, e, "scene upload");
    }

    ShadeScene& S = sc->view;
    S.trav.nodes = d_nodes;
    S.trav.tris = d_tris;
    S.trav.instances = d_inst;
    S.trav.lights = d_lights;
    S.trav.root = tlasRoot;
    S.trav.numLights = v->num_lights;
    S.trav.numNodes = (int)(recs.size() / 4);
    S.trav.numTris = v->num_tris;
    S.trav.numInstances = v->num_instances;
    S.trav.cullRel = 1.0e-4f;
    S.trav.cullAbs = 64.0f * ulp_of(extent);
    S.trav.wnodes = d_wide;
    S.trav.wroot = wroot;
    S.trav.wideOn = 1;
    S.trav.refNodes = d_refNodes;
    S.trav.refParent = d_parent;
    S.trav.leafOfTri = d_leafOfTri;
    S.trav.leafOfInst = d_leafOfInst;
    S.vertIndices = d_vidx;
    S.vertices = d_verts;
    S.normals = d_norms;
    S.materials = d_mats;
    S.inst = d_sinst;
    S.numMaterials = v->num_materials;
    S.shadeClassMask = shade_class_mask(sinst);
    if (hasEnv)
    {
        S.env.rgb = d_env;
        S.env.marginal = d_marg;
        S.env.cond = d_cond;
        S.env.w = v->env_width;
        S.env.h = v->env_height;
        S.env.resolution = (float)(v->env_width * v->env_height);
    }
    S.env.multiplier = 1.0f;
    if (hasTex)
    {
        S.tex.rgba = d_tex;
        S.tex.w = v->tex_width;
        S.tex.h = v->tex_height;
        S.tex.layers = v->num_textures;
    }
    sc->numRefNodes = v->num_nodes;
    sc->topLevelIndex = v->top_level_index;
    set_bounds(sc, nodes[v->top_level_index]);
    sc->d_nodes = d_nodes;
    sc->nodeCapacity = recs.size() / 4;
    sc->d_wide = d_wide;
    sc->wideCapacity = wideCap;
    sc->d_refNodes = d_refNodes;
    sc->d_parent = d_parent;
    sc->d_leafOfTri = d_leafOfTri;
    sc->d_leafOfInst = d_leafOfInst;
    sc->d_instances = d_inst;
    sc->d_sinst = d_sinst;
    sc->d_materials = d_mats;
    sc->numMaterials = v->num_materials;
    *out = sc;
    return LF_OK;
}

lf_status lf_scene_update_instances(lf_scene* sc, const lf_scene_view* v)
{
    if (!sc || !v) return LF_ERR_INVALID;
    lf_ctx* c = sc->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    if (v->num_nodes != sc->numRefNodes || v->top_level_index != sc->topLevelIndex ||
        v->num_instances != sc->view.trav.numInstances || v->num_materials != sc->numMaterials)
        return fail(c, LF_ERR_INVALID, "instance update must keep node, instance and material counts");
    // Re-encode everything host-side (mesh levels are unchanged, so the record count is
    // identical) and overwrite the node, instance and material arrays in place.
    const RefNode* nodes = reinterpret_cast<const RefNode*>(v->nodes);
    std::vector<float4> recs;
    recs.reserve(sc->nodeCapacity * 4);
    std::vector<int> map(v->num_nodes, -1);
    std::vector<float4> inst;
    std::vector<ShadeInstance> sinst;
    int tlasRoot = 0;
    lf_status st = encode_instances(c, v, nodes, recs, map, inst, sinst, &tlasRoot);
    if (st != LF_OK) return st;
    if (recs.size() / 4 > sc->nodeCapacity) return fail(c, LF_ERR_INVALID, "instance update grew the node array");
    std::vector<float4> wrecs;
    std::vector<int> parent, leafOfTri, leafOfInst;
    int wroot = 0;
    st = encode_wide(c, v, nodes, inst, wrecs, parent, leafOfTri, leafOfInst, &wroot);
    if (st != LF_OK) return st;
    if (wrecs.size() / kWideF4 > sc->wideCapacity) return fail(c, LF_ERR_INVALID, "instance update grew the wide tree");
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaMemcpy(sc->d_wide, wrecs.data(), wrecs.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(sc->d_refNodes, v->nodes, (size_t)v->num_nodes * 9 * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(sc->d_parent, parent.data(), parent.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(sc->d_leafOfTri, leafOfTri.data(), leafOfTri.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(sc->d_leafOfInst, leafOfInst.data(), leafOfInst.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(sc->d_nodes, recs.data(), recs.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(sc->d_instances, inst.data(), inst.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(sc->d_sinst, sinst.data(), sinst.size() * sizeof(ShadeInstance), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(sc->d_materials, v->materials, (size_t)v->num_materials * sizeof(DevMaterial), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(c, e, "instance update");
    sc->view.trav.root = tlasRoot;
    sc->view.trav.numNodes = (int)(recs.size() / 4);
    sc->view.trav.wroot = wroot;
    sc->view.shadeClassMask = shade_class_mask(sinst);
    set_bounds(sc, nodes[v->top_level_index]);
    return LF_OK;
}

lf_status lf_scene_release(lf_scene* sc)
{
    if (!sc) return LF_ERR_INVALID;
    if (sc->ctx)
    {
        cudaSetDevice(sc->ctx->device);
        cudaStreamSynchronize(sc->ctx->stream);
    }
    for (void* p : sc->allocs) cudaFree(p);
    delete sc;
    return LF_OK;
}

lf_status lf_scene_set_traversal(lf_scene* sc, int32_t wide)
{
    if (!sc || (wide != 0 && wide != 1)) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(sc->ctx->mu);
    cudaSetDevice(sc->ctx->device);
    cudaStreamSynchronize(sc->ctx->stream);
    sc->view.trav.wideOn = wide;
    return LF_OK;
}

lf_status lf_scene_set_culling(lf_scene* sc, float rel, float abs_margin)
{
    if (!sc) return LF_ERR_INVALID;
    sc->view.trav.cullRel = rel;
    sc->view.trav.cullAbs = abs_margin;
    return LF_OK;
}

size_t lf_scene_device_bytes(const lf_scene* sc) { return sc ? sc->bytes : 0; }

// ------------------------------------------------------------------ ray queries
}   // extern "C"

namespace
{
// Grows the binning scratch (keys, permutation, bin counters, fetch counter) of a context.
lf_status ensure_bin_scratch(lf_ctx* c, long long n)
{
    if (!c->binHist)
    {
        cudaError_t e = cudaMalloc((void**)&c->binHist, sizeof(uint32_t) * (size_t)trace_bins());
        if (e == cudaSuccess) e = cudaMalloc((void**)&c->binNext, sizeof(unsigned long long));
        if (e != cudaSuccess) return cuda_fail(c, e, "binning scratch");
    }
    if ((size_t)n > c->binCap)
    {
        cudaStreamSynchronize(c->stream);
        cudaFree(c->binKeys);
        cudaFree(c->binPerm);
        c->binKeys = nullptr;
        c->binPerm = nullptr;
        c->binCap = 0;
        cudaError_t e = cudaMalloc((void**)&c->binKeys, sizeof(uint32_t) * (size_t)n);
        if (e == cudaSuccess) e = cudaMalloc((void**)&c->binPerm, sizeof(int) * (size_t)n);
        if (e != cudaSuccess) return cuda_fail(c, e, "binning scratch");
        c->binCap = (size_t)n;
    }
    return LF_OK;
}
}

// Next event pair of the traversal-kernel timer (nullptr, nullptr when it is off).
void kernel_timer_pair(lf_ctx* c, cudaEvent_t* a, cudaEvent_t* b)
{
    *a = *b = nullptr;
    if (!c->kernelTimer) return;
    while (c->ktEvents.size() < 2 * (c->ktUsed + 1))
    {
        cudaEvent_t ev = nullptr;
        if (cudaEventCreate(&ev) != cudaSuccess) return;
        c->ktEvents.push_back(ev);
    }
    *a = c->ktEvents[2 * c->ktUsed];
    *b = c->ktEvents[2 * c->ktUsed + 1];
    ++c->ktUsed;
}

extern "C" {

lf_status lf_trace_closest_device(lf_ctx* c, lf_scene* sc, const void* d_rays, int64_t n, void* d_hits, uint32_t flags)
{
    if (!c || !sc || (n > 0 && (!d_rays || !d_hits)) || n < 0) return LF_ERR_INVALID;
    if (n == 0) return LF_OK;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    bool stats = (flags & LF_TRACE_STATS) != 0;
    if (stats) cudaMemsetAsync(c->d_stats, 0, 3 * sizeof(unsigned long long), c->stream);
    int e;
    if (!stats && !(flags & LF_TRACE_SIMPLE))
    {
        lf_status bs = ensure_bin_scratch(c, n);
        if (bs != LF_OK) return bs;
        cudaEvent_t k0, k1;
        kernel_timer_pair(c, &k0, &k1);
        e = launch_trace_binned(sc->view.trav, (const float4*)d_rays, n, d_hits, false, (flags & LF_TRACE_LIGHTS) ? 1 : 0,
                                sc->boundsLo, sc->boundsHi, !(flags & LF_TRACE_UNSORTED), c->binKeys, c->binHist,
                                c->binPerm, c->binNext, c->d_status, c->stream, k0, k1);
    }
    else
        e = launch_trace_closest(sc->view.trav, (const float4*)d_rays, n, (int4*)d_hits, (flags & LF_TRACE_LIGHTS) ? 1 : 0,
                                 stats, c->d_status, c->d_stats, c->stream);
    if (e) return cuda_fail(c, (cudaError_t)e, "trace launch");
    return LF_OK;
}

lf_status lf_trace_any_device(lf_ctx* c, lf_scene* sc, const void* d_rays, int64_t n, void* d_occ, uint32_t flags)
{
    if (!c || !sc || (n > 0 && (!d_rays || !d_occ)) || n < 0) return LF_ERR_INVALID;
    if (n == 0) return LF_OK;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    bool stats = (flags & LF_TRACE_STATS) != 0;
    if (stats) cudaMemsetAsync(c->d_stats, 0, 3 * sizeof(unsigned long long), c->stream);
    int e;
    if (!stats && !(flags & LF_TRACE_SIMPLE))
    {
        lf_status bs = ensure_bin_scratch(c, n);
        if (bs != LF_OK) return bs;
        cudaEvent_t k0, k1;
        kernel_timer_pair(c, &k0, &k1);
        e = launch_trace_binned(sc->view.trav, (const float4*)d_rays, n, d_occ, true, (flags & LF_TRACE_LIGHTS) ? 1 : 0,
                                sc->boundsLo, sc->boundsHi, !(flags & LF_TRACE_UNSORTED), c->binKeys, c->binHist,
                                c->binPerm, c->binNext, c->d_status, c->stream, k0, k1);
    }
    else
        e = launch_trace_any(sc->view.trav, (const float4*)d_rays, n, (uint8_t*)d_occ, (flags & LF_TRACE_LIGHTS) ? 1 : 0,
                             stats, c->d_status, c->d_stats, c->stream);
    if (e) return cuda_fail(c, (cudaError_t)e, "trace launch");
    return LF_OK;
}

}   // extern "C"

namespace
{
// Pieces of a host-buffer query: the setting, else two from 2^24 rays up and one below. A
// piece is sorted and traced on its own, so its bins are sparser: on 10.5M triangles a piece
// of 2^23 rays traces 2 % slower than 2^24 rays at once and one of 2^22 rays 5 % slower;
// two pieces hide half of the copy in and gain 1-2 %, four lose.
int host_chunks(const lf_ctx* c, int64_t n, uint32_t flags)
{
    if (flags & LF_TRACE_STATS) return 1;
    int k = c->hostChunks > 0 ? c->hostChunks : (n >= (int64_t(1) << 24) ? 2 : 1);
    k = std::max(1, std::min(k, lf_ctx::kMaxHostChunks));
    return n >= 1024 * (int64_t)k ? k : 1;
}

cudaError_t ensure_chunk_streams(lf_ctx* c)
{
    if (c->copyOut) return cudaSuccess;
    cudaError_t e = cudaStreamCreateWithFlags(&c->copyIn, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copyOut, cudaStreamNonBlocking);
    for (int k = 0; k < lf_ctx::kMaxHostChunks && e == cudaSuccess; ++k)
    {
        e = cudaEventCreateWithFlags(&c->chunkIn[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->chunkDone[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->chunkStart, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->chunkEnd, cudaEventDisableTiming);
    return e;
}

// Device address of [p, p + bytes) when the whole range lies in one page-locked block that
// lf_host_alloc of this context made and mapped, else null.
char* mapped_range(const lf_ctx* c, const void* p, size_t bytes)
{
    const char* q = (const char*)p;
    for (const auto& h : c->hostBlocks)
        if (h.dev && q >= h.host && bytes <= h.bytes && (size_t)(q - h.host) <= h.bytes - bytes)
            return h.dev + (q - h.host);
    return nullptr;
}

// Copies the rays in, traces them and copies the results out, in `host_chunks` pieces: piece k
// is copied in on copyIn, sorted and traced on the context stream once its copy is done, and
// copied out on copyOut once traced, so copies of some pieces overlap the tracing of others.
// When the results go to a mapped page-locked block of this context, the kernels write them
// there and nothing is copied out. The context stream waits for the copy streams, and the
// call returns after it.
template <class Launch>
lf_status trace_host(lf_ctx* c, lf_scene* sc, const float* rays, int64_t n, void* out, size_t outElem, uint32_t flags,
                     Launch launch)
{
    if (!c || !sc || n < 0 || (n > 0 && (!rays || !out))) return LF_ERR_INVALID;
    if (n == 0) return LF_OK;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    auto ensure = [&](void** buf, size_t* cap, size_t bytes) -> cudaError_t {
        if (*cap >= bytes) return cudaSuccess;
        cudaStreamSynchronize(c->stream);
        cudaFree(*buf);
        *buf = nullptr;
        *cap = 0;
        cudaError_t err = cudaMalloc(buf, bytes);
        if (err == cudaSuccess) *cap = bytes;
        return err;
    };
    char* direct = mapped_range(c, out, (size_t)n * outElem);
    cudaError_t e = ensure(&c->scratchRays, &c->scratchRaysBytes, (size_t)n * 32);
    if (e == cudaSuccess && !direct) e = ensure(&c->scratchOut, &c->scratchOutBytes, (size_t)n * outElem);
    const int K = host_chunks(c, n, flags);
    if (e == cudaSuccess && K > 1) e = ensure_chunk_streams(c);
    char* d_rays = (char*)c->scratchRays;
    char* d_out = direct ? direct : (char*)c->scratchOut;
    lf_status st = LF_OK;
    if (e == cudaSuccess && K == 1)
    {
        e = cudaMemcpyAsync(d_rays, rays, (size_t)n * 32, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) st = launch(d_rays, d_out, n);
        if (e == cudaSuccess && st == LF_OK && !direct)
            e = cudaMemcpyAsync(out, d_out, (size_t)n * outElem, cudaMemcpyDeviceToHost, c->stream);
    }
    else if (e == cudaSuccess)
    {
        // pieces of whole 1024-ray groups; the last takes the rest
        const int64_t step = ((n / K) + 1023) / 1024 * 1024;
        e = cudaEventRecord(c->chunkStart, c->stream);   // after earlier users of the scratch
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->copyIn, c->chunkStart, 0);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->copyOut, c->chunkStart, 0);
        for (int k = 0; k < K && e == cudaSuccess; ++k)
        {
            const int64_t lo = std::min(n, step * k), hi = k == K - 1 ? n : std::min(n, step * (k + 1));
            e = cudaMemcpyAsync(d_rays + lo * 32, (const char*)rays + lo * 32, (size_t)(hi - lo) * 32,
                                cudaMemcpyHostToDevice, c->copyIn);
            if (e == cudaSuccess) e = cudaEventRecord(c->chunkIn[k], c->copyIn);
        }
        for (int k = 0; k < K && e == cudaSuccess && st == LF_OK; ++k)
        {
            const int64_t lo = std::min(n, step * k), hi = k == K - 1 ? n : std::min(n, step * (k + 1));
            e = cudaStreamWaitEvent(c->stream, c->chunkIn[k], 0);
            if (e == cudaSuccess && hi > lo) st = launch(d_rays + lo * 32, d_out + lo * outElem, hi - lo);
            if (direct) continue;
            if (e == cudaSuccess && st == LF_OK) e = cudaEventRecord(c->chunkDone[k], c->stream);
            if (e == cudaSuccess && st == LF_OK) e = cudaStreamWaitEvent(c->copyOut, c->chunkDone[k], 0);
            if (e == cudaSuccess && st == LF_OK)
                e = cudaMemcpyAsync((char*)out + lo * outElem, d_out + lo * outElem, (size_t)(hi - lo) * outElem,
                                    cudaMemcpyDeviceToHost, c->copyOut);
        }
        // the context stream waits for both copy streams whatever happened above
        cudaEventRecord(c->chunkEnd, c->copyIn);
        cudaStreamWaitEvent(c->stream, c->chunkEnd, 0);
        cudaEventRecord(c->chunkEnd, c->copyOut);
        cudaStreamWaitEvent(c->stream, c->chunkEnd, 0);
    }
    if (e == cudaSuccess && st == LF_OK) st = check_device(c);
    else cudaStreamSynchronize(c->stream);   // no copy may still touch the caller's buffers
    if (e == cudaSuccess && st == LF_OK && (flags & LF_TRACE_STATS))
    {
        unsigned long long s[3];
        cudaMemcpy(s, c->d_stats, sizeof s, cudaMemcpyDeviceToHost);
        for (int k = 0; k < 3; ++k) c->lastStats[k] = s[k];
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "trace");
    return st;
}
}

extern "C" {

lf_status lf_ctx_set_host_chunks(lf_ctx* c, int32_t chunks)
{
    if (!c || chunks < 0 || chunks > lf_ctx::kMaxHostChunks) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    c->hostChunks = chunks;
    return LF_OK;
}

lf_status lf_trace_closest(lf_ctx* c, lf_scene* sc, const float* rays, int64_t n, lf_hit* hits, uint32_t flags)
{
    return trace_host(c, sc, rays, n, hits, sizeof(lf_hit), flags, [&](void* dr, void* dout, int64_t m) {
        return lf_trace_closest_device(c, sc, dr, m, dout, flags);
    });
}

lf_status lf_trace_any(lf_ctx* c, lf_scene* sc, const float* rays, int64_t n, uint8_t* occ, uint32_t flags)
{
    return trace_host(c, sc, rays, n, occ, 1, flags, [&](void* dr, void* dout, int64_t m) {
        return lf_trace_any_device(c, sc, dr, m, dout, flags);
    });
}

lf_status lf_trace_stats(const lf_ctx* c, uint64_t out3[3])
{
    if (!c || !out3) return LF_ERR_INVALID;
    for (int k = 0; k < 3; ++k) out3[k] = c->lastStats[k];
    return LF_OK;
}

// ------------------------------------------------------------------ frames
extern "C++" {
namespace lfrt
{
void fill_params(Params& P, const lf_render_params* p, const lf_scene* sc)
{
    std::memset(&P, 0, sizeof P);
    P.width = p->width;
    P.height = p->height;
    P.tileW = p->tile_width > 0 ? p->tile_width : p->width;
    P.tileH = p->tile_height > 0 ? p->tile_height : p->height;
    // TiledRenderer.cpp:232-233: 1 / (screen / tile), in float
    P.invNumTilesX = 1.0f / ((float)p->width / (float)P.tileW);
    P.invNumTilesY = 1.0f / ((float)p->height / (float)P.tileH);
    P.maxDepth = p->max_depth;
    P.rrEnabled = p->enable_rr;
    P.rrDepth = p->rr_depth;
    bool envData = sc->view.env.rgb != nullptr;
    P.constantBg = p->use_constant_bg;
    P.envOnMiss = (p->use_env_map && envData) ? 1 : 0;
    P.useEnv = (P.envOnMiss && !P.constantBg) ? 1 : 0;
    P.useLights = sc->view.trav.numLights > 0 ? 1 : 0;
    for (int k = 0; k < 3; ++k)
    {
        P.bg[k] = p->bg_color[k];
        P.cam_pos[k] = p->cam_position[k];
        P.cam_right[k] = p->cam_right[k];
        P.cam_up[k] = p->cam_up[k];
        P.cam_fwd[k] = p->cam_forward[k];
    }
    P.fov = p->cam_fov;
    P.focalDist = p->cam_focal_dist;
    P.aperture = p->cam_aperture;
    P.seed = p->seed;
    P.frameBase = p->frame_base;
    P.frameStride = 1;
    P.tileOrdinal = 0;
    P.hdrMultiplier = p->hdr_multiplier;
}
}
}   // extern "C++"

namespace
{

void free_frame_buffers(lf_frame* f)
{
    for (void* q : f->allocs) cudaFree(q);
    f->allocs.clear();
    f->cap = 0;
}

lf_status alloc_paths(lf_frame* f, long long cap)
{
    lf_ctx* c = f->ctx;
    size_t bytes = 0;
    cudaError_t e = cudaSuccess;
    auto A = [&](auto** p, size_t n) {
        if (e == cudaSuccess) e = dalloc(f->allocs, bytes, p, n);
    };
    A(&f->ps.o, cap);
    A(&f->ps.d, cap);
    A(&f->ps.T, cap);
    A(&f->ps.L, cap);
    A(&f->ps.A, cap);
    A(&f->ps.rng, cap);
    A(&f->ps.info, cap);
    A(&f->ps.luv, cap);
    A(&f->ps.hit, cap);
    A(&f->bb.queue[0], cap);
    A(&f->bb.queue[1], cap);
    A(&f->bb.count, 2);
    A(&f->bb.shadow, cap);
    A(&f->bb.shadowCount, 1);
    A(&f->bb.fetch, 2);
    if (e != cudaSuccess)
    {
        free_frame_buffers(f);
        return cuda_fail(c, e, "path state allocation");
    }
    f->cap = cap;
    return LF_OK;
}
}

lf_status lf_frame_create(lf_ctx* c, lf_scene* sc, const lf_render_params* p, uint32_t flags, lf_frame** out)
{
    if (!c || !sc || !p || !out) return LF_ERR_INVALID;
    *out = nullptr;
    if (p->width <= 0 || p->height <= 0 || p->max_depth < 0 || p->tile_width < 0 || p->tile_height < 0)
        return fail(c, LF_ERR_INVALID, "bad render parameters");
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    lf_frame* f = new lf_frame;
    f->ctx = c;
    f->scene = sc;
    f->flags = flags;
    f->W = p->width;
    f->H = p->height;
    fill_params(f->P, p, sc);
    f->numTilesX = (f->W + f->P.tileW - 1) / f->P.tileW;
    f->numTilesY = (f->H + f->P.tileH - 1) / f->P.tileH;
    // default batch: about 8M path slots
    long long tilePix = (long long)f->P.tileW * f->P.tileH;
    f->sppBatch = (int)std::max(1LL, std::min(64LL, (8LL << 20) / tilePix));
    size_t bytes = 0;
    unsigned long long* ctr = nullptr;
    cudaError_t e = dalloc(f->fixedAllocs, bytes, &f->accum, (size_t)f->W * f->H);
    if (e == cudaSuccess && (flags & LF_FRAME_FP64_ACCUM)) e = dalloc(f->fixedAllocs, bytes, &f->accum64, (size_t)f->W * f->H * 3);
    if (e == cudaSuccess) e = dalloc(f->fixedAllocs, bytes, &ctr, 4);
    f->bb.ctr = ctr;
    f->bb.status = c->d_status;
    // per-batch path state is allocated on first use (the engine has its own pool)
    lf_status st = e == cudaSuccess ? LF_OK : cuda_fail(c, e, "frame allocation");
    if (st != LF_OK)
    {
        for (void* q : f->fixedAllocs) cudaFree(q);
        delete f;
        return st;
    }
    cudaMemsetAsync(f->accum, 0, sizeof(float4) * (size_t)f->W * f->H, c->stream);
    if (f->accum64) cudaMemsetAsync(f->accum64, 0, sizeof(double) * (size_t)f->W * f->H * 3, c->stream);
    cudaMemsetAsync(ctr, 0, 4 * sizeof(unsigned long long), c->stream);
    *out = f;
    return LF_OK;
}

lf_status lf_frame_set_batch(lf_frame* f, int32_t spb)
{
    if (!f || spb < 0) return LF_ERR_INVALID;
    lf_ctx* c = f->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    long long tilePix = (long long)f->P.tileW * f->P.tileH;
    int want = spb == 0 ? (int)std::max(1LL, std::min(64LL, (8LL << 20) / tilePix)) : spb;
    if (want == f->sppBatch) return LF_OK;
    cudaStreamSynchronize(c->stream);
    free_frame_buffers(f);   // per-batch state is reallocated at the next batch
    if (f->graph)
    {
        cudaGraphExecDestroy(f->graph);
        f->graph = nullptr;
    }
    f->sppBatch = want;
    return LF_OK;
}

namespace
{
// Ends the capture begun by run_batch, updates (or instantiates) the frame's graph with the
// recorded batch and launches it.
lf_status end_batch_graph(lf_frame* f, cudaError_t launchErr, const char* what)
{
    lf_ctx* c = f->ctx;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (launchErr != cudaSuccess || e != cudaSuccess)
    {
        if (g) cudaGraphDestroy(g);
        return cuda_fail(c, launchErr != cudaSuccess ? launchErr : e, what);
    }
    if (f->graph)
    {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(f->graph, g, &info) != cudaSuccess)
        {
            cudaGetLastError();
            cudaGraphExecDestroy(f->graph);
            f->graph = nullptr;
        }
    }
    if (!f->graph) e = cudaGraphInstantiate(&f->graph, g, 0);
    cudaGraphDestroy(g);
    if (e == cudaSuccess) e = cudaGraphLaunch(f->graph, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "batch graph launch");
    return LF_OK;
}

// One batch of samples on one tile: generate, maxDepth bounces, accumulate. With a guide,
// `record` keeps the batch's path vertices and collects training samples.
lf_status run_batch(lf_frame* f, Params P, int firstSample, int n, bool record = false)
{
    lf_ctx* c = f->ctx;
    const ShadeScene& S = f->scene->view;
    ShadeScene Sv = S;
    Sv.env.multiplier = P.hdrMultiplier;
    long long tilePix = (long long)P.tileW * P.tileH;
    long long cap = (long long)n * tilePix;
    if (f->cap < cap)
    {
        free_frame_buffers(f);
        lf_status st = alloc_paths(f, (long long)std::max(n, f->sppBatch) * tilePix);
        if (st != LF_OK) return st;
    }
    const bool graph = (f->flags & LF_FRAME_USE_GRAPH) != 0;
    if (graph)
    {
        cudaError_t ce = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
        if (ce != cudaSuccess) return cuda_fail(c, ce, "batch graph capture");
    }
    cudaMemsetAsync(f->bb.count, 0, 2 * sizeof(int), c->stream);
    int e = launch_generate(Sv, P, f->ps, firstSample, n, f->bb.queue[0], f->bb.count, c->stream);
    if (e) return graph ? end_batch_graph(f, cudaErrorLaunchFailure, "generate launch")
                        : cuda_fail(c, (cudaError_t)e, "generate launch");
    BounceBuffers bb = f->bb;
    // Queue order is already coherent (camera rays in pixel order, survivors compacted in
    // order): warps take 32 queued rays at a time and trace each to its end.
    if (f->guide)
    {
        GuideBuffers gb = f->gb;
        gb.net = guide_net(f->guide);
        gb.tensorPath = guide_tensor_path(f->guide);
        gb.rec = record ? f->gb.rec : nullptr;
        for (int b = 0; b < P.maxDepth && !e; ++b) e = launch_bounce_guided(Sv, P, f->ps, bb, gb, b, cap, c->stream);
        if (!e && record)
        {
            cudaMemsetAsync(gb.trainCount, 0, sizeof(int), c->stream);
            e = launch_guide_collect(f->ps, gb, cap, c->stream);
        }
    }
    else
        for (int b = 0; b < P.maxDepth && !e; ++b) e = launch_bounce(Sv, P, f->ps, bb, b, cap, c->stream);
    if (!e) e = launch_accumulate(P, f->ps, n, f->accum, f->accum64, c->stream);
    f->lastBatchSamples = n;
    if (graph) return end_batch_graph(f, (cudaError_t)e, "batch launch");
    if (e) return cuda_fail(c, (cudaError_t)e, "batch launch");
    return LF_OK;
}
}

namespace
{
void free_guide_buffers(lf_frame* f)
{
    for (void* q : f->guideAllocs) cudaFree(q);
    f->guideAllocs.clear();
    f->guideCap = 0;
    f->gb = GuideBuffers{};
}

lf_status alloc_guide_buffers(lf_frame* f, long long cap)
{
    free_guide_buffers(f);
    size_t bytes = 0;
    cudaError_t e = cudaSuccess;
    auto A = [&](auto** q, size_t n) {
        if (e == cudaSuccess) e = dalloc(f->guideAllocs, bytes, q, n);
    };
    const int depth = std::max(1, f->P.maxDepth);
    A(&f->gb.queries, (size_t)cap * guide::kSampleFloats);
    A(&f->gb.mix, (size_t)cap * guide::kMixFloats);
    A(&f->gb.rec, (size_t)cap * depth * kGuideRecFloats);
    A(&f->gb.train, (size_t)f->guideTrainCap * guide::kSampleFloats);
    A(&f->gb.trainCount, 1);
    if (e != cudaSuccess)
    {
        free_guide_buffers(f);
        return cuda_fail(f->ctx, e, "guide buffers");
    }
    f->gb.trainCap = f->guideTrainCap;
    f->gb.alpha = f->guideAlpha;
    f->gb.maxDepth = depth;
    f->gb.weightClamp = 1e4f;
    f->guideCap = cap;
    return LF_OK;
}

// Guided batches of up to sppBatch samples (every tile); every train_every-th batch records
// its path vertices and trains the guide afterwards (Adam steps of guideBatch samples over
// what it collected).
lf_status frame_render_guided(lf_frame* f, Params P, int firstSample, int count)
{
    lf_ctx* c = f->ctx;
    const long long tilePix = (long long)P.tileW * P.tileH;
    const long long cap = (long long)std::max(1, f->sppBatch) * tilePix;
    if (f->guideCap < cap)
    {
        lf_status st = alloc_guide_buffers(f, cap);
        if (st != LF_OK) return st;
    }
    if (f->lastRadiance)
    {
        cudaFreeAsync(f->lastRadiance, c->stream);
        f->lastRadiance = nullptr;
        f->lastRadianceSamples = 0;
    }
    const bool tiledFrames = (f->flags & LF_FRAME_TILED_FRAMES) != 0;
    for (int s = 0; s < count;)
    {
        const int n = std::min(std::max(1, f->sppBatch), count - s);
        const bool record = f->guideTrainEvery > 0 && f->guideBatches % (uint64_t)f->guideTrainEvery == 0;
        ++f->guideBatches;
        for (int ty = f->numTilesY - 1; ty >= 0; --ty)
            for (int tx = 0; tx < f->numTilesX; ++tx)
            {
                P.tileX = tx;
                P.tileY = ty;
                P.tileOrdinal = tiledFrames ? (f->numTilesY - 1 - ty) * f->numTilesX + tx : 0;
                lf_status st = run_batch(f, P, firstSample + s, n, record);
                if (st != LF_OK) return st;
                if (!record) continue;
                int collected = 0;
                cudaError_t e = cudaMemcpyAsync(&collected, f->gb.trainCount, sizeof(int), cudaMemcpyDeviceToHost,
                                                c->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
                if (e != cudaSuccess) return cuda_fail(c, e, "guide sample count");
                const int avail = std::min(collected, f->gb.trainCap);
                const int steps = std::min(64, (avail + f->guideBatch - 1) / f->guideBatch);
                for (int k = 0; k < steps; ++k)
                {
                    const int off = k * f->guideBatch;
                    const int nb = std::min(f->guideBatch, avail - off);
                    st = lf_guide_train_device(f->guide, f->gb.train + (size_t)off * guide::kSampleFloats, nb,
                                               f->guideLr);
                    if (st != LF_OK) return st;
                    f->guideSteps++;
                    f->guideSamples += (uint64_t)nb;
                }
            }
        s += n;
    }
    return LF_OK;
}
}

lf_status lf_frame_render(lf_frame* f, int32_t first_sample, int32_t count)
{
    if (!f || count < 0 || first_sample < 0) return LF_ERR_INVALID;
    lf_ctx* c = f->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    Params P = f->P;
    const bool tiledFrames = (f->flags & LF_FRAME_TILED_FRAMES) != 0;
    P.frameStride = tiledFrames ? f->numTilesX * f->numTilesY : 1;
    if (f->guide)
    {
        if (count == 0) return LF_OK;
        lf_status st = frame_render_guided(f, P, first_sample, count);
        if (st == LF_OK) f->paths += (uint64_t)count * f->W * f->H;
        return st;
    }
    if (!(f->flags & LF_FRAME_PER_BATCH))
    {
        if (count == 0) return LF_OK;
        lf_status st = frame_render_engine(f, P, first_sample, count);
        if (st == LF_OK) f->paths += (uint64_t)count * f->W * f->H;
        return st;
    }
    if (f->lastRadiance)
    {
        cudaFreeAsync(f->lastRadiance, c->stream);
        f->lastRadiance = nullptr;
        f->lastRadianceSamples = 0;
    }
    int s = 0;
    while (s < count)
    {
        int n = std::min(f->sppBatch, count - s);
        for (int ty = f->numTilesY - 1; ty >= 0; --ty)      // TiledRenderer order: top tile row first
            for (int tx = 0; tx < f->numTilesX; ++tx)
            {
                P.tileX = tx;
                P.tileY = ty;
                P.tileOrdinal = tiledFrames ? (f->numTilesY - 1 - ty) * f->numTilesX + tx : 0;
                lf_status st = run_batch(f, P, first_sample + s, n);
                if (st != LF_OK) return st;
            }
        s += n;
    }
    f->paths += (uint64_t)count * f->W * f->H;
    return LF_OK;
}

lf_status lf_frame_render_tile(lf_frame* f, int32_t sample, int32_t tile_x, int32_t tile_y)
{
    if (!f || sample < 0 || tile_x < 0 || tile_y < 0 || tile_x >= f->numTilesX || tile_y >= f->numTilesY)
        return LF_ERR_INVALID;
    lf_ctx* c = f->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    Params P = f->P;
    const bool tiledFrames = (f->flags & LF_FRAME_TILED_FRAMES) != 0;
    P.frameStride = tiledFrames ? f->numTilesX * f->numTilesY : 1;
    P.tileX = tile_x;
    P.tileY = tile_y;
    P.tileOrdinal = tiledFrames ? (f->numTilesY - 1 - tile_y) * f->numTilesX + tile_x : 0;
    if (f->lastRadiance)
    {
        cudaFreeAsync(f->lastRadiance, c->stream);
        f->lastRadiance = nullptr;
        f->lastRadianceSamples = 0;
    }
    lf_status st = run_batch(f, P, sample, 1);
    if (st == LF_OK) f->paths += (uint64_t)f->P.tileW * f->P.tileH;
    return st;
}

lf_status lf_frame_sync(lf_frame* f)
{
    if (!f) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(f->ctx->mu);
    cudaSetDevice(f->ctx->device);
    return check_device(f->ctx);
}

lf_status lf_frame_read_accum(lf_frame* f, float* rgb)
{
    if (!f || !rgb) return LF_ERR_INVALID;
    lf_ctx* c = f->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    std::vector<float4> tmp((size_t)f->W * f->H);
    cudaError_t e = cudaMemcpyAsync(tmp.data(), f->accum, tmp.size() * sizeof(float4), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "accum readback");
    for (size_t i = 0; i < tmp.size(); ++i)
    {
        rgb[i * 3 + 0] = tmp[i].x;
        rgb[i * 3 + 1] = tmp[i].y;
        rgb[i * 3 + 2] = tmp[i].z;
    }
    return check_device(c);
}

lf_status lf_frame_read_accum64(lf_frame* f, double* rgb)
{
    if (!f || !rgb) return LF_ERR_INVALID;
    if (!f->accum64) return fail(f->ctx, LF_ERR_STATE, "frame was created without LF_FRAME_FP64_ACCUM");
    lf_ctx* c = f->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    cudaError_t e = cudaMemcpyAsync(rgb, f->accum64, sizeof(double) * (size_t)f->W * f->H * 3, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "accum64 readback");
    return check_device(c);
}

lf_status lf_frame_read_paths(lf_frame* f, float* rgb, int32_t max_samples)
{
    if (!f || !rgb || max_samples <= 0) return LF_ERR_INVALID;
    if (f->numTilesX * f->numTilesY != 1) return fail(f->ctx, LF_ERR_STATE, "path readback needs a single tile");
    lf_ctx* c = f->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    const float4* src = f->lastRadiance ? f->lastRadiance : f->ps.L;
    int n = std::min(max_samples, f->lastRadiance ? f->lastRadianceSamples : f->lastBatchSamples);
    if (!src || n <= 0) return fail(c, LF_ERR_STATE, "no rendered paths to read");
    const size_t pix = (size_t)f->W * f->H;
    // the engine's pass buffer is [sample][pixel]; the per-batch slots are [sample][tile
    // position] with the tile's pixels in pixel_of order
    const bool slots = !f->lastRadiance;
    const int tw = f->P.tileW, th = f->P.tileH;
    const size_t per = slots ? (size_t)tw * th : pix;
    std::vector<float4> tmp(per * n);
    cudaError_t e = cudaMemcpyAsync(tmp.data(), src, tmp.size() * sizeof(float4), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "path readback");
    for (int s = 0; s < n; ++s)
        for (size_t k = 0; k < per; ++k)
        {
            size_t i = k;
            if (slots)
            {
                int x, y;
                pixel_of((int)k, tw, th, x, y);
                if (x >= f->W || y >= f->H) continue;
                i = (size_t)y * f->W + x;
            }
            const float4 v = tmp[(size_t)s * per + k];
            float* d = rgb + ((size_t)s * pix + i) * 3;
            d[0] = v.x;
            d[1] = v.y;
            d[2] = v.z;
        }
    return check_device(c);
}

lf_status lf_frame_reset(lf_frame* f)
{
    if (!f) return LF_ERR_INVALID;
    lf_ctx* c = f->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    cudaMemsetAsync(f->accum, 0, sizeof(float4) * (size_t)f->W * f->H, c->stream);
    if (f->accum64) cudaMemsetAsync(f->accum64, 0, sizeof(double) * (size_t)f->W * f->H * 3, c->stream);
    cudaMemsetAsync(f->bb.ctr, 0, 4 * sizeof(unsigned long long), c->stream);
    f->paths = 0;
    return LF_OK;
}

lf_status lf_frame_counters(lf_frame* f, uint64_t out4[4])
{
    if (!f || !out4) return LF_ERR_INVALID;
    lf_ctx* c = f->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    unsigned long long v[4];
    cudaError_t e = cudaMemcpyAsync(v, f->bb.ctr, sizeof v, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "counter readback");
    for (int k = 0; k < 4; ++k) out4[k] = v[k];
    out4[0] = f->paths;
    return LF_OK;
}

lf_status lf_frame_set_guide(lf_frame* f, lf_guide* g, float alpha, int32_t train_every, float lr)
{
    if (!f || train_every < 0 || (g && !(alpha > 0.f && alpha < 1.f)) || (g && train_every > 0 && !(lr > 0.f)))
        return LF_ERR_INVALID;
    lf_ctx* c = f->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    f->guide = g;
    f->guideAlpha = alpha;
    f->guideTrainEvery = train_every;
    f->guideLr = lr;
    f->gb.alpha = alpha;
    if (!g) free_guide_buffers(f);
    return LF_OK;
}

lf_status lf_frame_guide_stats(lf_frame* f, uint64_t* steps, uint64_t* samples)
{
    if (!f || !steps || !samples) return LF_ERR_INVALID;
    *steps = f->guideSteps;
    *samples = f->guideSamples;
    return LF_OK;
}

lf_status lf_frame_release(lf_frame* f)
{
    if (!f) return LF_ERR_INVALID;
    cudaSetDevice(f->ctx->device);
    cudaStreamSynchronize(f->ctx->stream);
    if (f->lastRadiance)
    {
        cudaFreeAsync(f->lastRadiance, f->ctx->stream);
        cudaStreamSynchronize(f->ctx->stream);
    }
    if (f->engineJob >= 0 && f->ctx->engine) engine_job_free(f->ctx->engine, f->engineJob);
    free_guide_buffers(f);
    if (f->graph) cudaGraphExecDestroy(f->graph);
    for (void* q : f->allocs) cudaFree(q);
    for (void* q : f->fixedAllocs) cudaFree(q);
    delete f;
    return LF_OK;
}
}

// ------------------------------------------------------------------ engine configuration
extern "C" {
lf_status lf_ctx_configure_engine(lf_ctx* c, int32_t slots, int32_t block_extend, int32_t block_shade,
                                  int32_t block_shadow, int32_t shade_threads_per_sm)
{
    if (!c) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    EngineHost* e = nullptr;
    lf_status st = engine_get(c, &e);
    if (st != LF_OK) return st;
    return engine_configure(e, slots, block_extend, block_shade, block_shadow, shade_threads_per_sm);
}

lf_status lf_ctx_set_engine_drain(lf_ctx* c, int64_t paths)
{
    if (!c || paths < 0) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    EngineHost* e = nullptr;
    lf_status st = engine_get(c, &e);
    if (st != LF_OK) return st;
    e->drainPaths = paths;
    return LF_OK;
}

lf_status lf_ctx_set_engine_sort(lf_ctx* c, int32_t sort_by_material)
{
    if (!c || sort_by_material < 0 || sort_by_material > 2) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    EngineHost* e = nullptr;
    lf_status st = engine_get(c, &e);
    if (st != LF_OK) return st;
    return engine_set_sort(e, sort_by_material);
}

lf_status lf_ctx_engine_info(lf_ctx* c, int64_t* slots, int64_t* device_bytes)
{
    if (!c || !slots || !device_bytes) return LF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    *slots = c->engine ? c->engine->b.cap : 0;
    *device_bytes = c->engine ? (int64_t)c->engine->poolBytes : 0;
    return LF_OK;
}
}

// ------------------------------------------------------------------ render without allocating
// Some callers cannot allocate device memory at render time: plugin hosts that hand the
// renderer a fixed device arena and account for every byte on the GPU themselves, and
// real-time loops that forbid allocation inside a frame (cudaMalloc and cudaFree can
// synchronise the device and stall the frame, and may fail once another allocator holds the
// memory). lf_render_noalloc serves them: all wavefront state lives in one file-scope device
// array of fixed size, and the accumulation buffer is the caller's.
namespace
{
constexpr long long kNoAllocPaths = 131072;   // path slots = max pixels of one tile
constexpr size_t kNoAllocAlign = 256;
constexpr size_t kNoAllocHeader = 256;        // queue sizes, status word, counters
constexpr size_t noalloc_round(size_t b) { return (b + kNoAllocAlign - 1) / kNoAllocAlign * kNoAllocAlign; }
// PathSoA: o, d, T, L, A, rng, info, hit (16 B each), luv (8 B); two int queues; next-event records
constexpr size_t kNoAllocBytes = kNoAllocHeader + 8 * noalloc_round(kNoAllocPaths * 16) +
                                 noalloc_round(kNoAllocPaths * 8) + 2 * noalloc_round(kNoAllocPaths * 4) +
                                 noalloc_round(kNoAllocPaths * sizeof(ShadowRec));
}

// 30 MiB + 256 B (31.5 MB) on every GPU that loads the library, kept until the process exits.
static_assert(kNoAllocBytes == 30ull * 1024 * 1024 + 256, "documented size of the no-alloc scratch array");
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace
{
std::mutex g_noalloc_mu;
void* g_noalloc_addr[64] = {};

// Device address of the scratch array for the current device; resolved once per device.
lf_status noalloc_base(lf_ctx* c, unsigned char** base)
{
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (c->device < 0 || c->device >= 64) return fail(c, LF_ERR_INVALID, "device index out of range");
    if (!g_noalloc_addr[c->device])
    {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return cuda_fail(c, e, "cudaGetSymbolAddress(no-alloc scratch)");
        g_noalloc_addr[c->device] = p;
    }
    *base = static_cast<unsigned char*>(g_noalloc_addr[c->device]);
    return LF_OK;
}
}

extern "C" lf_status lf_render_noalloc(lf_scene* sc, const lf_render_params* p, int32_t first_sample, int32_t count,
                                       void* d_accum)
{
    if (!sc || !p || !d_accum || count < 0 || first_sample < 0) return LF_ERR_INVALID;
    lf_ctx* c = sc->ctx;
    if (p->width <= 0 || p->height <= 0 || p->max_depth < 0 || p->tile_width < 0 || p->tile_height < 0)
        return fail(c, LF_ERR_INVALID, "bad render parameters");
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    Params P;
    fill_params(P, p, sc);
    const long long tilePix = (long long)P.tileW * P.tileH;
    if (tilePix > kNoAllocPaths)
        return fail(c, LF_ERR_INVALID, "lf_render_noalloc: a tile of " + std::to_string(P.tileW) + "x" +
                                           std::to_string(P.tileH) + " pixels exceeds the fixed capacity of " +
                                           std::to_string(kNoAllocPaths) + " paths; set tile_width/tile_height");
    if (count == 0) return LF_OK;
    unsigned char* base = nullptr;
    lf_status st = noalloc_base(c, &base);
    if (st != LF_OK) return st;

    // carve the scratch array
    unsigned char* q = base + kNoAllocHeader;
    auto take = [&](size_t bytes) {
        unsigned char* r = q;
        q += noalloc_round(bytes);
        return r;
    };
    const size_t N = (size_t)kNoAllocPaths;
    PathSoA ps;
    ps.o = (float4*)take(N * 16);
    ps.d = (float4*)take(N * 16);
    ps.T = (float4*)take(N * 16);
    ps.L = (float4*)take(N * 16);
    ps.A = (float4*)take(N * 16);
    ps.rng = (uint4*)take(N * 16);
    ps.info = (int4*)take(N * 16);
    ps.hit = (float4*)take(N * 16);
    ps.luv = (float2*)take(N * 8);
    BounceBuffers bb;
    bb.queue[0] = (int*)take(N * 4);
    bb.queue[1] = (int*)take(N * 4);
    bb.shadow = (ShadowRec*)take(N * sizeof(ShadowRec));
    bb.count = (int*)(base + 0);
    bb.shadowCount = (int*)(base + 8);
    bb.status = (uint32_t*)(base + 12);
    bb.ctr = (unsigned long long*)(base + 16);
    bb.fetch = (unsigned long long*)(base + 48);

    // the array keeps the previous call's contents: clear sizes, status and counters
    cudaError_t e = cudaMemsetAsync(base, 0, kNoAllocHeader, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "no-alloc scratch clear");

    ShadeScene Sv = sc->view;
    Sv.env.multiplier = P.hdrMultiplier;
    const int numTilesX = (P.width + P.tileW - 1) / P.tileW, numTilesY = (P.height + P.tileH - 1) / P.tileH;
    const int spb = (int)std::max(1LL, std::min<long long>(64, kNoAllocPaths / tilePix));
    for (int s = 0; s < count;)
    {
        int n = std::min(spb, count - s);
        for (int ty = numTilesY - 1; ty >= 0; --ty)
            for (int tx = 0; tx < numTilesX; ++tx)
            {
                P.tileX = tx;
                P.tileY = ty;
                long long cap = (long long)n * tilePix;
                cudaMemsetAsync(bb.count, 0, 2 * sizeof(int), c->stream);
                int le = launch_generate(Sv, P, ps, first_sample + s, n, bb.queue[0], bb.count, c->stream);
                for (int b = 0; le == 0 && b < P.maxDepth; ++b) le = launch_bounce(Sv, P, ps, bb, b, cap, c->stream);
                if (le == 0) le = launch_accumulate(P, ps, n, (float4*)d_accum, nullptr, c->stream);
                if (le) return cuda_fail(c, (cudaError_t)le, "no-alloc render launch");
            }
        s += n;
    }
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "no-alloc render");
    uint32_t bits = 0;
    e = cudaMemcpy(&bits, bb.status, sizeof bits, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "no-alloc status readback");
    if (bits)
    {
        c->devErrors |= bits;
        return fail(c, LF_ERR_DEVICE, "device error bits 0x" + std::to_string(bits));
    }
    return LF_OK;
}
