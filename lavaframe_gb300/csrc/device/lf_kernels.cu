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
#include "lf_kernels.h"
#include "lf_shade.cuh"

namespace lfd
{
namespace
{
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ void set_error(uint32_t* status, uint32_t bits)
{
    if (bits && status) atomicOr(status, bits);
}

// Appends `item` for lanes with `pred`; one atomic per warp. All 32 lanes must call.
template <class T>
__device__ __forceinline__ void warp_push(bool pred, const T& item, T* queue, int* count, int cap, uint32_t* status)
{
    unsigned m = __ballot_sync(kFull, pred);
    if (!m) return;
    int lane = threadIdx.x & 31;
    int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(kFull, base, leader);
    if (pred)
    {
        int pos = base + __popc(m & ((1u << lane) - 1u));
        if (pos < cap) queue[pos] = item;
        else set_error(status, LF_DEVERR_QUEUE);
    }
}

__device__ __forceinline__ v3 f3(float4 a) { return v3(a.x, a.y, a.z); }
__device__ __forceinline__ float4 f4(v3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

__device__ __forceinline__ float map_range(float value, float low1, float high1, float low2, float high2)
{
    return low2 + ((value - low1) * (high2 - low2)) / (high1 - low1);
}
}

// ------------------------------------------------------------------ generate
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
            int lx = lp % P.tileW, ly = lp / P.tileW;
            int gx = P.tileX * P.tileW + lx, gy = P.tileY * P.tileH + ly;
            bool inside = gx < P.width && gy < P.height;
            ps.L[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
            ps.info[slot] = make_int4(inside ? gy * P.width + gx : -1, 0, 0, 0);
            if (inside)
            {
                // renderer.glsl:27-62
                float tcx = ((float)lx + 0.5f) / (float)P.tileW;
                float tcy = ((float)ly + 0.5f) / (float)P.tileH;
                float xoffset = -1.0f + 2.0f * P.invNumTilesX * (float)P.tileX;
                float yoffset = -1.0f + 2.0f * P.invNumTilesY * (float)P.tileY;
                float ctx = map_range(tcx, 0.0f, 1.0f, xoffset, xoffset + 2.0f * P.invNumTilesX);
                float cty = map_range(tcy, 0.0f, 1.0f, yoffset, yoffset + 2.0f * P.invNumTilesY);
                float fsx = map_range(tcx, 0.0f, 1.0f, P.invNumTilesX * (float)P.tileX,
                                      P.invNumTilesX * (float)P.tileX + P.invNumTilesX);
                float fsy = map_range(tcy, 0.0f, 1.0f, P.invNumTilesY * (float)P.tileY,
                                      P.invNumTilesY * (float)P.tileY + P.invNumTilesY);
                float px = fsx * (float)P.width, py = fsy * (float)P.height;
                uint32_t frame = (uint32_t)(P.frameBase + (firstSample + s) * P.frameStride + P.tileOrdinal);
                Rng rng;
                rng.x = (uint32_t)px;
                rng.y = (uint32_t)py;
                rng.z = frame;
                rng.w = (uint32_t)px + (uint32_t)py + P.seed * 0x9E3779B9u;

                float r1 = 2.0f * rnd(rng);
                float r2 = 2.0f * rnd(rng);
                float jx = r1 < 1.0f ? sqrtf(r1) - 1.0f : 1.0f - sqrtf(2.0f - r1);
                float jy = r2 < 1.0f ? sqrtf(r2) - 1.0f : 1.0f - sqrtf(2.0f - r2);
                jx = jx / ((float)P.width * 0.5f);
                jy = jy / ((float)P.height * 0.5f);
                float dx = ctx + jx, dy = cty + jy;
                float scale = lfc::tan_c(P.fov * 0.5f);
                dy = dy * ((float)P.height / (float)P.width * scale);
                dx = dx * scale;
                v3 right(P.cam_right[0], P.cam_right[1], P.cam_right[2]);
                v3 up(P.cam_up[0], P.cam_up[1], P.cam_up[2]);
                v3 fwd(P.cam_fwd[0], P.cam_fwd[1], P.cam_fwd[2]);
                v3 rayDir = lfc::normalize(dx * right + dy * up + fwd);
                v3 focalPoint = P.focalDist * rayDir;
                float cam_r1 = rnd(rng) * kTWO_PI;
                float cam_r2 = rnd(rng) * P.aperture;
                float sr, cr;
                lfc::sincos_c(cam_r1, &sr, &cr);
                v3 aperturePos = (cr * right + sr * up) * sqrtf(cam_r2);
                v3 dir = lfc::normalize(focalPoint - aperturePos);
                v3 org = v3(P.cam_pos[0], P.cam_pos[1], P.cam_pos[2]) + aperturePos;

                ps.o[slot] = f4(org, 0.0f);
                ps.d[slot] = f4(dir, 0.0f);
                ps.T[slot] = make_float4(1.f, 1.f, 1.f, 0.f);
                ps.A[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
                ps.rng[slot] = make_uint4(rng.x, rng.y, rng.z, rng.w);
                ps.luv[slot] = make_float2(0.f, 0.f);
                push = true;
            }
        }
        warp_push(push, slot, queue, qcount, (int)n, nullptr);
    }
}

// ------------------------------------------------------------------ extend
__global__ void extend_kernel(ShadeScene S, Params P, PathSoA ps, const int* queue, const int* qcount,
                              uint32_t* status, unsigned long long* ctr)
{
    const int n = *qcount;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ctr[1], (unsigned long long)n);
    const bool lights = P.useLights != 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        int p = queue[i];
        float4 o4 = ps.o[p], d4 = ps.d[p];
        Hit h;
        uint32_t err = closest_hit<false>(S.trav, f3(o4), f3(d4), kInfinity, lights, &h, nullptr);
        ps.hit[p] = make_float4(h.t, __int_as_float(h.inst), __int_as_float(h.prim), __int_as_float(h.light));
        set_error(status, err);
    }
}

// ------------------------------------------------------------------ shade
__global__ void shade_kernel(ShadeScene S, Params P, PathSoA ps, const int* qin, const int* qinCount, int* qout,
                             int* qoutCount, ShadowRec* sq, int* sqCount, int cap, uint32_t* status,
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
            float4 o4 = ps.o[p], d4 = ps.d[p], T4 = ps.T[p], L4 = ps.L[p], A4 = ps.A[p], h = ps.hit[p];
            int4 info = ps.info[p];
            uint4 r4 = ps.rng[p];
            Rng rng{r4.x, r4.y, r4.z, r4.w};
            v3 o = f3(o4), d = f3(d4), T = f3(T4), L = f3(L4), A = f3(A4);
            float bsdfPdf = o4.w;
            const int depth = info.y;
            const float t = h.x;
            const int inst = __float_as_int(h.y), prim = __float_as_int(h.z), light = __float_as_int(h.w);

            if (t == kInfinity)
            {
                if (P.constantBg)
                    L = L + v3(P.bg[0], P.bg[1], P.bg[2]) * T;
                else if (P.envOnMiss)
                {
                    float mis = 1.0f;
                    v3 col = env_lookup(S.env, d);
                    if (depth > 0)
                    {
                        float lightPdf = EnvPdf(S.env, d);
                        mis = powerHeuristic(bsdfPdf, lightPdf);
                    }
                    L = L + mis * col * T * S.env.multiplier;
                }
                ps.L[p] = f4(L, 0.f);
            }
            else if (light >= 0)
            {
                // Analytic light: the shader still adds the emission of the material held
                // in the (stale) state from the last triangle hit before EmitterSample.
                v3 em = material_emission(S, info.z, lfc::v2(ps.luv[p].x, ps.luv[p].y));
                L = L + em * T;
                const DevLight& Lt = S.trav.lights[light];
                v3 Le(Lt.emission[0], Lt.emission[1], Lt.emission[2]);
                if (depth != 0)
                {
                    float lpdf;
                    if (Lt.type == 0.f)
                    {
                        float cosTheta = lfc::dot(-d, v3(Lt.normal[0], Lt.normal[1], Lt.normal[2]));
                        lpdf = (t * t) / (Lt.area * cosTheta);
                    }
                    else
                        lpdf = (t * t) / Lt.area;
                    Le = powerHeuristic(bsdfPdf, lpdf) * Le;
                }
                L = L + Le * T;
                ps.L[p] = f4(L, 0.f);
            }
            else
            {
                // ---- GetNormalsAndTexCoord (pathtrace.glsl:16-37)
                float m[12];
                int root, matId;
                load_instance(S.trav.instances + (size_t)inst * 4, m, &root, &matId);
                const ShadeInstance& SI = S.inst[inst];
                v3 ro = xform(m, o, 1.0f), rd = xform(m, d, 0.0f);
                float u, v;
                tri_hit(S.trav.tris + (size_t)prim * 3, ro, rd, &u, &v);
                float bw = 1.0f - u - v;
                v3 fhp = xform(SI.fwd, ro + rd * t, 1.0f);
                int4 vi = S.vertIndices[prim];
                float4 n1 = S.normals[vi.x], n2 = S.normals[vi.y], n3 = S.normals[vi.z];
                float w0 = S.vertices[vi.x].w, w1 = S.vertices[vi.y].w, w2 = S.vertices[vi.z].w;
                Surf s;
                s.texCoord = lfc::v2(w0, n1.w) * bw + lfc::v2(w1, n2.w) * u + lfc::v2(w2, n3.w) * v;
                v3 nrm = lfc::normalize(f3(n1) * bw + f3(n2) * u + f3(n3) * v);
                nrm = lfc::normalize(lfc::mul3(SI.nrm, nrm));
                s.normal = nrm;
                s.ffnormal = lfc::dot(nrm, d) <= 0.0f ? nrm : nrm * -1.0f;
                Onb(s.normal, s.tangent, s.bitangent);
                // ---- GetMaterialsAndTextures (pathtrace.glsl:40-123)
                s.mat = load_material(S, SI.material);
                apply_textures(S, s, d);
                s.eta = lfc::dot(d, s.normal) < 0.0f ? (1.0f / s.mat.ior) : s.mat.ior;
                info.z = SI.material;
                ps.luv[p] = make_float2(s.texCoord.x, s.texCoord.y);

                if (lfc::dot(s.normal, s.ffnormal) > 0.0f) A = v3(0.0f);
                L = L + s.mat.emission * T;
                T = T * lfc::vexp(-A * t);

                // ---- DirectLight (pathtrace.glsl:126-204): candidates, visibility later
                BsdfCtx bc{s.eta, s.mat, s.tangent, s.bitangent};
                v3 V = -d;
                v3 surfacePos = fhp + s.normal * kEps;
                uint32_t flags = 0;
                v3 envDir(0.f), envC(0.f), lightDir(0.f), lightC(0.f);
                float lightMax = 0.f;
                if (P.useEnv)
                {
                    v3 color;
                    float4 dp = EnvSample(S.env, rng, color);
                    envDir = v3(dp.x, dp.y, dp.z);
                    float lightPdf = dp.w;
                    float pdf;
                    v3 f = DisneyEval(bc, V, s.ffnormal, envDir, pdf);
                    if (pdf > 0.0f)
                    {
                        float mis = powerHeuristic(lightPdf, pdf);
                        if (mis > 0.0f)
                        {
                            envC = mis * f * fabsf(lfc::dot(envDir, s.ffnormal)) * color / lightPdf;
                            flags |= 1u;
                        }
                    }
                }
                if (P.useLights)
                {
                    const int nl = S.trav.numLights;
                    int li = (int)(rnd(rng) * (float)nl);
                    if (li >= nl)
                    {
                        li = nl - 1;
                        atomicAdd(&ctr[3], 1ull);
                    }
                    const DevLight& Lt = S.trav.lights[li];
                    v3 lpos(Lt.pos[0], Lt.pos[1], Lt.pos[2]);
                    v3 ldir, lnrm;
                    float ldist, lpdf;
                    v3 lem = v3(Lt.emission[0], Lt.emission[1], Lt.emission[2]) * (float)nl;
                    int type = (int)Lt.type;
                    if (type == 0 || type == 1)
                    {
                        float r1 = rnd(rng);
                        float r2 = rnd(rng);
                        v3 lsp;
                        if (type == 0)
                            lsp = lpos + v3(Lt.u[0], Lt.u[1], Lt.u[2]) * r1 + v3(Lt.v[0], Lt.v[1], Lt.v[2]) * r2;
                        else
                            lsp = lpos + UniformSampleSphere(r1, r2) * Lt.radius;
                        ldir = lsp - surfacePos;
                        ldist = lfc::length(ldir);
                        float distSq = ldist * ldist;
                        ldir = ldir / ldist;
                        lnrm = type == 0 ? v3(Lt.normal[0], Lt.normal[1], Lt.normal[2]) : lfc::normalize(lsp - lpos);
                        lpdf = distSq / (Lt.area * fabsf(lfc::dot(lnrm, ldir)));
                    }
                    else
                    {
                        ldir = lfc::normalize(lpos - v3(0.0f));
                        lnrm = lfc::normalize(surfacePos - lpos);
                        ldist = kInfinity;
                        lpdf = 1.0f;
                    }
                    if (lfc::dot(ldir, lnrm) < 0.0f)
                    {
                        float pdf;
                        v3 f = DisneyEval(bc, V, s.ffnormal, ldir, pdf);
                        float weight = 1.0f;
                        if (Lt.area > 0.0f) weight = powerHeuristic(lpdf, pdf);
                        if (pdf > 0.0f)
                        {
                            lightC = weight * f * fabsf(lfc::dot(s.ffnormal, ldir)) * lem / lpdf;
                            lightDir = ldir;
                            lightMax = ldist - kEps;
                            flags |= 2u;
                        }
                    }
                }
                if (flags)
                {
                    rec.a = f4(surfacePos, __int_as_float(p));
                    rec.b = f4(T, __uint_as_float(flags));
                    rec.c = f4(envDir, 0.f);
                    rec.e = f4(envC, 0.f);
                    rec.f = f4(lightDir, lightMax);
                    rec.g = f4(lightC, 0.f);
                    pushShadow = true;
                }
                else
                    L = L + v3(0.0f) * T;

                // ---- DisneySample, absorption, throughput, RR (pathtrace.glsl:268-291)
                v3 Ls;
                float pdf;
                v3 f = DisneySample(bc, rng, V, s.ffnormal, Ls, pdf);
                if (lfc::dot(s.ffnormal, Ls) < 0.0f) A = (-lfc::vlog(s.mat.extinction)) / s.mat.atDistance;
                bool alive = true;
                if (pdf > 0.0f)
                    T = T * (f * fabsf(lfc::dot(s.ffnormal, Ls)) / pdf);
                else
                    alive = false;
                if (alive && P.rrEnabled && depth >= P.rrDepth)
                {
                    float q = lfc::fmin_g(lfc::fmax_g(T.x, lfc::fmax_g(T.y, T.z)) + 0.001f, 0.95f);
                    if (rnd(rng) > q) alive = false;
                    else T = T / q;
                }
                if (alive)
                {
                    d = Ls;
                    o = fhp + d * kEps;
                    if (depth + 1 < P.maxDepth) pushExt = true;
                }
                info.y = depth + 1;
                ps.o[p] = f4(o, pdf);
                ps.d[p] = f4(d, 0.f);
                ps.T[p] = f4(T, 0.f);
                ps.L[p] = f4(L, 0.f);
                ps.A[p] = f4(A, 0.f);
                ps.rng[p] = make_uint4(rng.x, rng.y, rng.z, rng.w);
                ps.info[p] = info;
            }
        }
        warp_push(pushExt, p, qout, qoutCount, cap, status);
        warp_push(pushShadow, rec, sq, sqCount, cap, status);
    }
}

// ------------------------------------------------------------------ shadow
__global__ void shadow_kernel(ShadeScene S, Params P, PathSoA ps, const ShadowRec* sq, const int* sqCount,
                              uint32_t* status, unsigned long long* ctr)
{
    const int n = *sqCount;
    const bool lights = P.useLights != 0;
    unsigned long long rays = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        ShadowRec rec = sq[i];
        int p = __float_as_int(rec.a.w);
        uint32_t flags = __float_as_uint(rec.b.w);
        v3 pos = f3(rec.a);
        v3 Li(0.0f);
        Hit h;
        bool occ;
        uint32_t err = 0;
        if (flags & 1u)
        {
            err |= any_hit<false>(S.trav, pos, f3(rec.c), kInfinity - kEps, lights, &occ, &h, nullptr);
            if (!occ) Li = Li + f3(rec.e);
            ++rays;
        }
        if (flags & 2u)
        {
            err |= any_hit<false>(S.trav, pos, f3(rec.f), rec.f.w, lights, &occ, &h, nullptr);
            if (!occ) Li = Li + f3(rec.g);
            ++rays;
        }
        float4 L4 = ps.L[p];
        v3 L = f3(L4) + Li * f3(rec.b);
        ps.L[p] = f4(L, 0.f);
        set_error(status, err);
    }
    if (rays) atomicAdd(&ctr[2], rays);
}

// ------------------------------------------------------------------ persistent extend / shadow
// Same work as extend_kernel / shadow_kernel, organised like the batched ray queries: warps
// stay resident, and a lane whose ray finished takes the next queue entry (one atomic per
// warp refill), so long rays do not hold a whole warp of finished lanes.
__global__ void __launch_bounds__(128) extend_persistent_kernel(ShadeScene S, Params P, PathSoA ps, const int* queue,
                                                                 const int* qcount, unsigned long long* fetch,
                                                                 uint32_t* status, unsigned long long* ctr)
{
    const int n = *qcount;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ctr[1], (unsigned long long)n);
    const int lane = threadIdx.x & 31;
    TravState s;
    int p = -1;          // -1: needs work, -2: queue exhausted
    int light = -1;
    while (true)
    {
        unsigned need = __ballot_sync(kFull, p == -1);
        if (need)
        {
            int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(fetch, (unsigned long long)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            if (p == -1)
            {
                unsigned long long my = base + __popc(need & ((1u << lane) - 1u));
                if (my < (unsigned long long)n)
                {
                    p = queue[my];
                    v3 o = f3(ps.o[p]), d = f3(ps.d[p]);
                    float t = kInfinity;
                    light = -1;
                    if (P.useLights) t = lights_closest(S.trav, o, d, t, &light);
                    trav_init(s, S.trav, o, d, t);
                }
                else
                    p = -2;
            }
        }
        if (__all_sync(kFull, p == -2)) break;
        if (p >= 0 && trav_run<false>(s, S.trav, 32))
        {
            ps.hit[p] = make_float4(s.t, __int_as_float(s.hitInst), __int_as_float(s.hitPrim),
                                    __int_as_float(s.hitPrim >= 0 ? -1 : light));
            set_error(status, s.err);
            p = -1;
        }
    }
}

__global__ void __launch_bounds__(128) shadow_persistent_kernel(ShadeScene S, Params P, PathSoA ps, const ShadowRec* sq,
                                                                 const int* sqCount, unsigned long long* fetch,
                                                                 uint32_t* status, unsigned long long* ctr)
{
    const int n = *sqCount;
    const int lane = threadIdx.x & 31;
    TravState s;
    int r = -1;          // record index; -1: needs work, -2: exhausted
    int phase = 0;       // 0: environment ray, 1: light ray, 2: done
    bool tracing = false;
    v3 Li(0.0f);
    unsigned long long rays = 0;
    while (true)
    {
        unsigned need = __ballot_sync(kFull, r == -1);
        if (need)
        {
            int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(fetch, (unsigned long long)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            if (r == -1)
            {
                unsigned long long my = base + __popc(need & ((1u << lane) - 1u));
                r = my < (unsigned long long)n ? (int)my : -2;
                phase = 0;
                tracing = false;
                Li = v3(0.0f);
            }
        }
        if (__all_sync(kFull, r == -2)) break;
        if (r < 0) continue;
        if (!tracing)
        {
            const uint32_t flags = __float_as_uint(sq[r].b.w);
            while (phase < 2 && !(flags & (1u << phase))) ++phase;
            if (phase == 2)
            {
                // DirectLight's Li, then radiance += Li * throughput (pathtrace.glsl:266)
                const int p = __float_as_int(sq[r].a.w);
                v3 L = f3(ps.L[p]) + Li * f3(sq[r].b);
                ps.L[p] = f4(L, 0.f);
                r = -1;
                continue;
            }
            const v3 pos = f3(sq[r].a);
            const float4 dir4 = phase == 0 ? sq[r].c : sq[r].f;
            const float maxd = phase == 0 ? kInfinity - kEps : sq[r].f.w;
            const v3 dir = f3(dir4);
            ++rays;
            if (P.useLights && lights_any(S.trav, pos, dir, maxd))
            {
                ++phase;   // occluded by an analytic light
                continue;
            }
            trav_init(s, S.trav, pos, dir, maxd);
            tracing = true;
        }
        if (trav_run<true>(s, S.trav, 32))
        {
            if (s.hitPrim < 0) Li = Li + (phase == 0 ? f3(sq[r].e) : f3(sq[r].g));
            set_error(status, s.err);
            tracing = false;
            ++phase;
        }
    }
    if (rays) atomicAdd(&ctr[2], rays);
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
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
    if (per_sm <= 0) per_sm = 1;
    long long full = (long long)g_num_sms * per_sm;
    long long need = (work + block - 1) / block;
    if (need < 1) need = 1;
    return (int)(need < full ? need : full);
}
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
    if (b.fetch)
    {
        cudaMemsetAsync(b.fetch, 0, 2 * sizeof(unsigned long long), st);
        int ge = grid_for((const void*)extend_persistent_kernel, BE, cap);
        extend_persistent_kernel<<<ge, BE, 0, st>>>(S, P, ps, qin, cin, b.fetch, b.status, b.ctr);
    }
    else
    {
        int ge = grid_for((const void*)extend_kernel, BE, cap);
        extend_kernel<<<ge, BE, 0, st>>>(S, P, ps, qin, cin, b.status, b.ctr);
    }
    int gs = grid_for((const void*)shade_kernel, BS, cap);
    shade_kernel<<<gs, BS, 0, st>>>(S, P, ps, qin, cin, qout, cout, b.shadow, b.shadowCount, (int)cap, b.status, b.ctr);
    if (b.fetch)
    {
        int gw = grid_for((const void*)shadow_persistent_kernel, BW, cap);
        shadow_persistent_kernel<<<gw, BW, 0, st>>>(S, P, ps, b.shadow, b.shadowCount, b.fetch + 1, b.status, b.ctr);
    }
    else
    {
        int gw = grid_for((const void*)shadow_kernel, BW, cap);
        shadow_kernel<<<gw, BW, 0, st>>>(S, P, ps, b.shadow, b.shadowCount, b.status, b.ctr);
    }
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
