// Per-path steps of the wavefront pipeline, shared by the per-batch frame kernels
// (lf_kernels.cu) and the persistent multi-job engine (lf_engine.cu): camera ray generation,
// surface / miss / emitter shading with next-event candidates, and next-event visibility.
#pragma once

#include "lf_guide.cuh"
#include "lf_kernels.h"
#include "lf_pixel.h"

namespace lfd
{
namespace pathops
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

// Appends `item` for threads with `pred`; one atomic per block. Every thread of the block
// must call (it synchronises the block); `smem` holds at least blockDim.x / 32 + 1 ints.
template <class T>
__device__ __forceinline__ void block_push(bool pred, const T& item, T* queue, int* count, int cap,
                                           uint32_t* status, int* smem)
{
    const unsigned m = __ballot_sync(kFull, pred);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0) smem[warp] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0)
    {
        int tot = 0;
        for (int w = 0; w < nw; ++w)
        {
            const int c = smem[w];
            smem[w] = tot;
            tot += c;
        }
        smem[nw] = tot ? atomicAdd(count, tot) : 0;
    }
    __syncthreads();
    if (pred)
    {
        const int pos = smem[nw] + smem[warp] + __popc(m & ((1u << lane) - 1u));
        if (pos < cap) queue[pos] = item;
        else set_error(status, LF_DEVERR_QUEUE);
    }
    __syncthreads();
}

// counter += v summed over the warp, one atomic per warp. All 32 lanes must call.
__device__ __forceinline__ void warp_count_add(unsigned long long* counter, unsigned long long v)
{
    const unsigned s = __reduce_add_sync(kFull, (unsigned)v);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(counter, (unsigned long long)s);
}

__device__ __forceinline__ v3 f3(float4 a) { return v3(a.x, a.y, a.z); }
__device__ __forceinline__ float4 f4(v3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

__device__ __forceinline__ float map_range(float value, float low1, float high1, float low2, float high2)
{
    return low2 + ((value - low1) * (high2 - low2)) / (high1 - low1);
}
}

// Camera ray of one path into `slot` (renderer.glsl:27-62): tile-local pixel (lx, ly) of tile
// (tileX, tileY), sample index `sample`, frame number frameBase + sample * frameStride +
// tileOrdinal. Resets the per-path state.
__device__ __forceinline__ void gen_path(const Params& P, int tileX, int tileY, int tileOrdinal, int sample, int lx,
                                         int ly, const PathSoA& ps, int slot)
{
    using namespace pathops;
    // renderer.glsl:27-62
    float tcx = ((float)lx + 0.5f) / (float)P.tileW;
    float tcy = ((float)ly + 0.5f) / (float)P.tileH;
    float xoffset = -1.0f + 2.0f * P.invNumTilesX * (float)tileX;
    float yoffset = -1.0f + 2.0f * P.invNumTilesY * (float)tileY;
    float ctx = map_range(tcx, 0.0f, 1.0f, xoffset, xoffset + 2.0f * P.invNumTilesX);
    float cty = map_range(tcy, 0.0f, 1.0f, yoffset, yoffset + 2.0f * P.invNumTilesY);
    float fsx = map_range(tcx, 0.0f, 1.0f, P.invNumTilesX * (float)tileX,
                          P.invNumTilesX * (float)tileX + P.invNumTilesX);
    float fsy = map_range(tcy, 0.0f, 1.0f, P.invNumTilesY * (float)tileY,
                          P.invNumTilesY * (float)tileY + P.invNumTilesY);
    float px = fsx * (float)P.width, py = fsy * (float)P.height;
    uint32_t frame = (uint32_t)(P.frameBase + sample * P.frameStride + tileOrdinal);
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
}

// Position and interpolated shading normal (before normal mapping) of a triangle hit, as in
// GetNormalsAndTexCoord (pathtrace.glsl:16-37).
struct SurfaceGeom
{
    v3 fhp;          // world hit point
    v3 nrm;          // world shading normal
    lfc::v2 texCoord;
    int material;
};

__device__ __forceinline__ SurfaceGeom surface_geom(const ShadeScene& S, v3 o, v3 d, float t, int inst, int prim)
{
    float m[12];
    int root, matId;
    load_instance(S.trav.instances + (size_t)inst * 4, m, &root, &matId);
    const ShadeInstance& SI = S.inst[inst];
    v3 ro = xform(m, o, 1.0f), rd = xform(m, d, 0.0f);
    float u, v;
    tri_hit(S.trav.tris + (size_t)prim * 3, ro, rd, &u, &v);
    float bw = 1.0f - u - v;
    SurfaceGeom g;
    g.fhp = xform(SI.fwd, ro + rd * t, 1.0f);
    int4 vi = S.vertIndices[prim];
    float4 n1 = S.normals[vi.x], n2 = S.normals[vi.y], n3 = S.normals[vi.z];
    float w0 = S.vertices[vi.x].w, w1 = S.vertices[vi.y].w, w2 = S.vertices[vi.z].w;
    g.texCoord = lfc::v2(w0, n1.w) * bw + lfc::v2(w1, n2.w) * u + lfc::v2(w2, n3.w) * v;
    v3 nrm = lfc::normalize(pathops::f3(n1) * bw + pathops::f3(n2) * u + pathops::f3(n3) * v);
    g.nrm = lfc::normalize(lfc::mul3(SI.nrm, nrm));
    g.material = SI.material;
    return g;
}

// Guided sampling state of one bounce (learned path guiding; no reference counterpart).
// mix: the mixture of each queue position; rec: per path slot, maxDepth training records of
// kGuideRecFloats (hit point, outgoing direction, normal, sampled direction, pdf, throughput
// after the vertex, radiance at the next vertex's start, state), stored field-major - field k
// of vertex d of slot p at (d * kGuideRecFloats + k) * recStride + p - so that a warp's
// neighbouring slots write and read neighbouring words.
struct GuideCtx
{
    const float* mix;
    float* rec;
    float alpha;     // probability of sampling the mixture instead of the BSDF
    int maxDepth;
    long long recStride;   // path slots of the batch
};

__device__ __forceinline__ float* guide_rec(float* rec, long long stride, int p, int depth, int k)
{
    return rec + ((size_t)depth * kGuideRecFloats + k) * (size_t)stride + p;
}

// One bounce of PathTrace for the path in slot p after its closest hit is known
// (pathtrace.glsl:208-294 minus the visibility tests): returns whether the path continues
// (pushExt) and whether it has next-event rays (pushShadow, described by rec).
// kGuided: directions come from the learned mixture with probability alpha and from the BSDF
// otherwise (one-sample MIS: the pdf is alpha * p_mix + (1 - alpha) * p_bsdf, the BSDF value
// DisneyEval's), the same combined pdf weighs next-event estimation, and the vertex is
// recorded for training; qpos is the path's queue position (index of its mixture).
// kLights = false compiles the analytic-light code out, for scenes without lights (no ray can
// then hit a light, and next-event estimation samples the environment only).
template <bool kGuided, bool kLights = true>
__device__ __forceinline__ void shade_path_t(const ShadeScene& S, const Params& P, const PathSoA& ps, int p,
                                             unsigned long long* ctr, bool& pushExt, bool& pushShadow, ShadowRec& rec,
                                             const GuideCtx& gc, int qpos)
{
    using namespace pathops;
    float4 o4 = ps.o[p], d4 = ps.d[p], T4 = ps.T[p], L4 = ps.L[p], A4 = ps.A[p], h = ps.hit[p];
    int4 info = ps.info[p];
    uint4 r4 = ps.rng[p];
    Rng rng{r4.x, r4.y, r4.z, r4.w};
    v3 o = f3(o4), d = f3(d4), T = f3(T4), L = f3(L4), A = f3(A4);
    float bsdfPdf = o4.w;
    const int depth = info.y;
    const float t = h.x;
    const int inst = __float_as_int(h.y), prim = __float_as_int(h.z), light = __float_as_int(h.w);
    if (kGuided && gc.rec && depth > 0)
    {
        // radiance at the start of this vertex: everything the previous vertex's direction
        // has not carried yet
        *guide_rec(gc.rec, gc.recStride, p, depth - 1, 16) = L.x;
        *guide_rec(gc.rec, gc.recStride, p, depth - 1, 17) = L.y;
        *guide_rec(gc.rec, gc.recStride, p, depth - 1, 18) = L.z;
        *guide_rec(gc.rec, gc.recStride, p, depth - 1, 19) = 2.f;
    }

    if (t == kInfinity)
    {
        if (P.constantBg)
            L = L + v3(P.bg[0], P.bg[1], P.bg[2]) * T;
        else if (P.envOnMiss)
        {
            const v3 mc = env_miss_term(S.env, d, depth, bsdfPdf);
            L = L + mc * T * S.env.multiplier;
        }
        ps.L[p] = f4(L, 0.f);
    }
    else if (kLights && light >= 0)
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
        const SurfaceGeom geo = surface_geom(S, o, d, t, inst, prim);
        const v3 fhp = geo.fhp;
        const v3 nrm = geo.nrm;
        Surf s;
        s.texCoord = geo.texCoord;
        s.normal = nrm;
        s.ffnormal = lfc::dot(nrm, d) <= 0.0f ? nrm : nrm * -1.0f;
        Onb(s.normal, s.tangent, s.bitangent);
        // ---- GetMaterialsAndTextures (pathtrace.glsl:40-123)
        s.mat = load_material(S, geo.material);
        if (has_texture_maps(s.mat)) s = apply_texture_maps(S, s, d);
        s.eta = lfc::dot(d, s.normal) < 0.0f ? (1.0f / s.mat.ior) : s.mat.ior;
        info.z = geo.material;
        const float* mix = kGuided ? gc.mix + (size_t)qpos * guide::kMixFloats : nullptr;
        const float alpha = kGuided ? gc.alpha : 0.f;
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
                const float dirPdf =
                    kGuided ? alpha * guide::mix_pdf(mix, envDir.x, envDir.y, envDir.z) + (1.0f - alpha) * pdf : pdf;
                float mis = powerHeuristic(lightPdf, dirPdf);
                if (mis > 0.0f)
                {
                    envC = mis * f * fabsf(lfc::dot(envDir, s.ffnormal)) * color / lightPdf;
                    flags |= 1u;
                }
            }
        }
        if (kLights && P.useLights)
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
                const float dirPdf =
                    kGuided ? alpha * guide::mix_pdf(mix, ldir.x, ldir.y, ldir.z) + (1.0f - alpha) * pdf : pdf;
                if (Lt.area > 0.0f) weight = powerHeuristic(lpdf, dirPdf);
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
        v3 f;
        if (kGuided)
        {
            if (rnd(rng) < alpha)
            {
                const float u0 = rnd(rng), u1 = rnd(rng), u2 = rnd(rng);
                guide::mix_sample(mix, u0, u1, u2, &Ls.x, &Ls.y, &Ls.z);
            }
            else
                DisneySample(bc, rng, V, s.ffnormal, Ls, pdf);
            float bsdfPdfL;
            f = DisneyEval(bc, V, s.ffnormal, Ls, bsdfPdfL);
            pdf = alpha * guide::mix_pdf(mix, Ls.x, Ls.y, Ls.z) + (1.0f - alpha) * bsdfPdfL;
        }
        else
            f = DisneySample(bc, rng, V, s.ffnormal, Ls, pdf);
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
        if (kGuided && gc.rec && depth < gc.maxDepth)
        {
            const float vals[16] = {fhp.x, fhp.y, fhp.z, V.x, V.y, V.z, nrm.x, nrm.y, nrm.z,
                                    Ls.x,  Ls.y,  Ls.z,  pdf, T.x, T.y, T.z};
#pragma unroll
            for (int k = 0; k < 16; ++k) *guide_rec(gc.rec, gc.recStride, p, depth, k) = vals[k];
            *guide_rec(gc.rec, gc.recStride, p, depth, 19) = pushExt ? 1.f : 0.f;
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

template <bool kLights = true>
__device__ __forceinline__ void shade_path(const ShadeScene& S, const Params& P, const PathSoA& ps, int p,
                                           unsigned long long* ctr, bool& pushExt, bool& pushShadow, ShadowRec& rec)
{
    shade_path_t<false, kLights>(S, P, ps, p, ctr, pushExt, pushShadow, rec, GuideCtx{nullptr, nullptr, 0.f, 0, 0}, 0);
}

// Visibility of a path's next-event rays, then radiance += Li * throughput
// (pathtrace.glsl:126-204, 266). Returns device error bits; counts traced rays. The record is
// read field by field where it is used (a queued record in global memory, or the drain's own),
// so that only the position, the path, the flags and Li stay live across the traversals.
// `Lout`, when given, receives the path's radiance as written.
__device__ __forceinline__ uint32_t shadow_path(const ShadeScene& S, const Params& P, const PathSoA& ps,
                                                const ShadowRec* rec, unsigned long long& rays,
                                                float4* Lout = nullptr)
{
    using namespace pathops;
    const bool lights = P.useLights != 0;
    const float4 a4 = rec->a;
    const int p = __float_as_int(a4.w);
    const uint32_t flags = __float_as_uint(rec->b.w);
    const v3 pos = f3(a4);
    v3 Li(0.0f);
    Hit h;
    bool occ;
    uint32_t err = 0;
    // the record's rays in order (environment first, then the light), through one traversal
    // call site, so that lanes trace their first rays together
    const int nr = __popc(flags & 3u);
    for (int j = 0; j < nr; ++j)
    {
        const bool env = (flags & 1u) && j == 0;
        const float4 dir = env ? rec->c : rec->f;
        err |= any_hit<false>(S.trav, pos, f3(dir), env ? kInfinity - kEps : dir.w, lights, &occ, &h, nullptr);
        if (!occ)
        {
            const float4 col = env ? rec->e : rec->g;
            Li = Li + f3(col);
        }
        ++rays;
    }
    const float4 T4 = rec->b;
    float4 L4 = ps.L[p];
    v3 L = f3(L4) + Li * f3(T4);
    ps.L[p] = f4(L, 0.f);
    if (Lout) *Lout = f4(L, 0.f);
    return err;
}
}
