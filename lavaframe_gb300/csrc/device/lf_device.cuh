// Device-side scene layout and software BVH traversal (GB300 has no RT cores).
//
// Layout in HBM (built from the reference flat arrays by the upload code):
//  - inner nodes, 64 B each (4 x float4), both children's boxes in one record:
//      f0 = (Lmin.xyz, Lmax.x) f1 = (Lmax.yz, Rmin.xy) f2 = (Rmin.z, Rmax.xyz)
//      f3 = (left code, right code, -, -)
//    A child code >= 0 is an inner-node record; < 0 is a leaf, ~code being
//    (first packed triangle << 2 | count) on the mesh level and the instance index on the
//    instance level. One 64 B load replaces the reference's three texel fetches per node
//    plus two per child box (closest_hit.glsl:102,169-170).
//  - triangles in packed (leaf) order, 48 B each: v0, e0 = v1 - v0, e1 = v2 - v0
//    (the reference forms the same differences per test, closest_hit.glsl:119-120).
//  - instances, 64 B: inverse transform columns 0..3 (xyz) + mesh root code + material;
//    the reference inverts the 4x4 at every instance-leaf visit (closest_hit.glsl:159-160).
//  - lights, precomputed plane/normal/scaled edges (closest_hit.glsl:30-35).
//
// Traversal keeps the reference's visit order exactly: nearer child first by the value
// AABBIntersect returns (t0, or t1 when the origin is inside; ties go left), a sentinel
// separating the instance and mesh levels, strict `t < tBest` acceptance, and the stack
// capacity of 64 (overflow ends the ray and raises LF_DEVERR_STACK instead of writing past
// the array). Optional culling skips a child whose entry distance max(t0, 0) exceeds the
// best hit so far by a safety margin; it never changes which triangle wins except when
// rounding puts a triangle in front of its own box by more than the margin.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../../include/lavaframe_gb300.h"
#include "../lf_vec.h"

namespace lfd
{
using lfc::v3;

constexpr float kInfinity = 1000000.0f;   // INFINITY in shaders/common/globals.glsl:8
constexpr float kEps = 0.001f;            // EPS in globals.glsl:9
constexpr int kStackSize = 64;            // stack[64] in closest_hit.glsl:70
constexpr int kStackCap = 63;             // one slot of the 64 holds the bottom sentinel
constexpr int kMaxTraversalSteps = 1 << 22;

// Device error bits (LF_DEVERR_*) are the ones of the C ABI, OR-ed into a status word.

struct DevLight
{
    float pos[3], emission[3], u[3], v[3];
    float radius, area, type;
    float normal[3];        // normalize(cross(u, v))
    float planeW;           // dot(normal, pos)
    float us[3], vs[3];     // u / dot(u,u), v / dot(v,v)
    float pad[3];
};

// Wide nodes collapsed from the reference's binary tree (see traverse_wide): per node
// 2 * kWide float4 = [min x | max x | min y | max y | min z | max z | child codes | child
// reference-node indices], kWide values per group (kWide / 4 float4 each); unused slots have
// code kWideEmpty and the empty box lo = +inf, hi = -inf (no slab test passes it: wide_slabs
// reads it as entry +inf, exit -inf). The width is a build option
// (LF_WIDE = 4 or 8).
#ifndef LF_WIDE
#define LF_WIDE 4
#endif
constexpr int kWide = LF_WIDE;
static_assert(kWide == 4 || kWide == 8, "wide nodes have 4 or 8 children");
constexpr int kWideF4 = 2 * kWide;
constexpr int kWideEmpty = (int)0x80000002;
constexpr int kWideStack = kWide == 8 ? 160 : 96;

struct DevScene
{
    const float4* nodes;        // 4 float4 per inner node
    const float4* tris;         // 3 float4 per packed triangle
    const float4* instances;    // 4 float4 per instance
    const DevLight* lights;
    int root;                   // instance-level root code
    int numLights;
    int numNodes, numTris, numInstances;
    float cullRel;              // relative culling margin, < 0 disables culling
    float cullAbs;              // absolute culling margin (a few ulps of the scene extent)
    // wide traversal (null wnodes or wideOn == 0: binary traversal everywhere)
    const float4* wnodes;       // kWideF4 float4 per wide node
    int wroot;                  // instance-level root code in the wide tree
    int wideOn;
    const float* refNodes;      // the reference's 36-byte nodes, for tie resolution
    const int* refParent;       // parent of every reference node, -1 at roots
    const int* leafOfTri;       // reference leaf node of every packed triangle
    const int* leafOfInst;      // reference instance-level leaf node of every instance
};

struct TraceStats
{
    unsigned long long nodes, tris, leaves;
};

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

// AABBIntersect (intersection.glsl:53-68) returning both the reference's value and the
// entry distance used for culling.
__device__ __forceinline__ float box_hit(float bminx, float bminy, float bminz, float bmaxx, float bmaxy,
                                         float bmaxz, v3 o, v3 invd, float* entry)
{
    float fx = (bmaxx - o.x) * invd.x, fy = (bmaxy - o.y) * invd.y, fz = (bmaxz - o.z) * invd.z;
    float nx = (bminx - o.x) * invd.x, ny = (bminy - o.y) * invd.y, nz = (bminz - o.z) * invd.z;
    float tmaxx = lfc::fmax_g(fx, nx), tmaxy = lfc::fmax_g(fy, ny), tmaxz = lfc::fmax_g(fz, nz);
    float tminx = lfc::fmin_g(fx, nx), tminy = lfc::fmin_g(fy, ny), tminz = lfc::fmin_g(fz, nz);
    float t1 = lfc::fmin_g(tmaxx, lfc::fmin_g(tmaxy, tmaxz));
    float t0 = lfc::fmax_g(tminx, lfc::fmax_g(tminy, tminz));
    *entry = t0 > 0.f ? t0 : 0.f;
    return (t1 >= t0) ? (t0 > 0.f ? t0 : t1) : -1.0f;
}

// The exact test for rays with a zero, denormal or non-finite inverse direction component:
// their slab values can be NaN or infinite, so the entry is no lower bound of the hit distance
// and such rays are never culled.
__device__ __forceinline__ float box_hit_exact(float bminx, float bminy, float bminz, float bmaxx, float bmaxy,
                                               float bmaxz, v3 o, v3 invd, float* entry)
{
    const float h = box_hit(bminx, bminy, bminz, bmaxx, bmaxy, bmaxz, o, invd, entry);
    *entry = 0.f;
    return h;
}

// Three-input min / max (sm_100 and later).
__device__ __forceinline__ float fmin3_hw(float a, float b, float c)
{
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

__device__ __forceinline__ float fmax3_hw(float a, float b, float c)
{
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// The same test for rays whose inverse direction is finite and non-zero in every component.
// Then no slab value is NaN (no 0 * inf), and the hardware min / max agree with the GLSL
// select forms except for the sign of a zero result, which no comparison below can see
// (t0 and t1 are only compared with each other and with zero, the returned value only with
// zero and the sibling's value, the entry only with a positive limit). Rays with a zero or
// denormal direction component keep the exact form.
__device__ __forceinline__ float box_hit_fast(float bminx, float bminy, float bminz, float bmaxx, float bmaxy,
                                              float bmaxz, v3 o, v3 invd, float* entry)
{
    float fx = (bmaxx - o.x) * invd.x, fy = (bmaxy - o.y) * invd.y, fz = (bmaxz - o.z) * invd.z;
    float nx = (bminx - o.x) * invd.x, ny = (bminy - o.y) * invd.y, nz = (bminz - o.z) * invd.z;
    float t1 = fmin3_hw(fmaxf(fx, nx), fmaxf(fy, ny), fmaxf(fz, nz));
    float t0 = fmax3_hw(fminf(fx, nx), fminf(fy, ny), fminf(fz, nz));
    *entry = fmaxf(t0, 0.f);
    return (t1 >= t0) ? (t0 > 0.f ? t0 : t1) : -1.0f;
}

__device__ __forceinline__ bool fast_inv(float x) { return fabsf(x) < 3.0e38f && x != 0.f; }   // false for NaN

// Inverse direction and whether the fast box test applies to it.
__device__ __forceinline__ v3 inv_dir(v3 d, bool* fast)
{
    // __frcp_rn is the correctly rounded reciprocal: the same bits as the IEEE division 1.0f / x
    v3 inv(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
    *fast = fast_inv(inv.x) && fast_inv(inv.y) && fast_inv(inv.z);
    return inv;
}

// Both child boxes of an inner-node record.
__device__ __forceinline__ void box_pair(float4 f0, float4 f1, float4 f2, v3 o, v3 invd, bool fast, float* hL,
                                         float* hR, float* eL, float* eR)
{
    if (fast)
    {
        *hL = box_hit_fast(f0.x, f0.y, f0.z, f0.w, f1.x, f1.y, o, invd, eL);
        *hR = box_hit_fast(f1.z, f1.w, f2.x, f2.y, f2.z, f2.w, o, invd, eR);
    }
    else
    {
        *hL = box_hit_exact(f0.x, f0.y, f0.z, f0.w, f1.x, f1.y, o, invd, eL);
        *hR = box_hit_exact(f1.z, f1.w, f2.x, f2.y, f2.z, f2.w, o, invd, eR);
    }
}

// Moller-Trumbore as in closest_hit.glsl:119-134: returns t (= uvt.z) when all of
// (u, v, t, 1-u-v) are >= 0, else a negative value. u, v returned for barycentrics.
__device__ __forceinline__ float tri_hit(const float4* tri, v3 o, v3 d, float* pu, float* pv)
{
    float4 a = ldg4(tri + 0), b = ldg4(tri + 1), c = ldg4(tri + 2);
    v3 v0(a.x, a.y, a.z), e0(b.x, b.y, b.z), e1(c.x, c.y, c.z);
    v3 p = lfc::cross(d, e1);
    float det = lfc::dot(e0, p);
    v3 tv = o - v0;
    v3 q = lfc::cross(tv, e0);
    float ux = lfc::dot(tv, p) / det;
    float uy = lfc::dot(d, q) / det;
    float uz = lfc::dot(e1, q) / det;
    float uw = 1.0f - ux - uy;
    *pu = ux;
    *pv = uy;
    bool ok = ux >= 0.0f && uy >= 0.0f && uz >= 0.0f && uw >= 0.0f;
    return ok ? uz : -1.0f;
}

// tri_hit for a hit that only counts at distances in [0, tmax]: the distance quotient is formed
// first and the two barycentric quotients only when it is in range. Each quotient is the same
// IEEE division as in tri_hit, so a hit is reported exactly when tri_hit reports it with
// t <= tmax.
__device__ __forceinline__ float tri_hit_upto(const float4* tri, v3 o, v3 d, float tmax)
{
    float4 a = ldg4(tri + 0), b = ldg4(tri + 1), c = ldg4(tri + 2);
    v3 v0(a.x, a.y, a.z), e0(b.x, b.y, b.z), e1(c.x, c.y, c.z);
    v3 p = lfc::cross(d, e1);
    float det = lfc::dot(e0, p);
    v3 tv = o - v0;
    v3 q = lfc::cross(tv, e0);
    float uz = lfc::dot(e1, q) / det;
    if (!(uz >= 0.0f && uz <= tmax)) return -1.0f;
    float ux = lfc::dot(tv, p) / det;
    float uy = lfc::dot(d, q) / det;
    float uw = 1.0f - ux - uy;
    bool ok = ux >= 0.0f && uy >= 0.0f && uw >= 0.0f;
    return ok ? uz : -1.0f;
}

// Instance inverse transform applied like `vec3(inverse(M) * vec4(x, w))`.
__device__ __forceinline__ void load_instance(const float4* rec, float m[12], int* root, int* mat)
{
    float4 a = ldg4(rec + 0), b = ldg4(rec + 1), c = ldg4(rec + 2), e = ldg4(rec + 3);
    m[0] = a.x; m[1] = a.y; m[2] = a.z; m[3] = a.w;
    m[4] = b.x; m[5] = b.y; m[6] = b.z; m[7] = b.w;
    m[8] = c.x; m[9] = c.y; m[10] = c.z; m[11] = c.w;
    *root = __float_as_int(e.x);
    *mat = __float_as_int(e.y);
}

// columns: c0 = m[0..2], c1 = m[3..5], c2 = m[6..8], c3 = m[9..11]
__device__ __forceinline__ v3 xform(const float m[12], v3 p, float w)
{
    return v3(m[0] * p.x + m[3] * p.y + m[6] * p.z + m[9] * w,
              m[1] * p.x + m[4] * p.y + m[7] * p.z + m[10] * w,
              m[2] * p.x + m[5] * p.y + m[8] * p.z + m[11] * w);
}

struct Hit
{
    float t;
    int inst;      // instance index, -1 if none
    int prim;      // packed triangle index, -1 if none
    int light;     // light index when an analytic light is the closest hit, else -1
};

// RectIntersect / SphereIntersect (intersection.glsl:7-50).
__device__ __forceinline__ float rect_intersect(const DevLight& L, v3 o, v3 d)
{
    v3 n(L.normal[0], L.normal[1], L.normal[2]);
    float dt = lfc::dot(d, n);
    float t = (L.planeW - lfc::dot(n, o)) / dt;
    if (t > kEps)
    {
        v3 p = o + d * t;
        v3 vi = p - v3(L.pos[0], L.pos[1], L.pos[2]);
        float a1 = lfc::dot(v3(L.us[0], L.us[1], L.us[2]), vi);
        if (a1 >= 0.f && a1 <= 1.f)
        {
            float a2 = lfc::dot(v3(L.vs[0], L.vs[1], L.vs[2]), vi);
            if (a2 >= 0.f && a2 <= 1.f)
                return t;
        }
    }
    return kInfinity;
}

__device__ __forceinline__ float sphere_intersect(const DevLight& L, v3 o, v3 d)
{
    v3 op = v3(L.pos[0], L.pos[1], L.pos[2]) - o;
    float eps = 0.001f;
    float b = lfc::dot(op, d);
    float det = b * b - lfc::dot(op, op) + L.radius * L.radius;
    if (det < 0.f) return kInfinity;
    det = sqrtf(det);
    float t1 = b - det;
    if (t1 > eps) return t1;
    float t2 = b + det;
    if (t2 > eps) return t2;
    return kInfinity;
}

// Shared two-level traversal. kAny: stop at the first triangle with t < tMax
// (anyhit.glsl:7-173); otherwise keep the closest (closest_hit.glsl:69-201).
// Returns device error bits (0 on success).
template <bool kAny, bool kStats>
__device__ __forceinline__ uint32_t traverse(const DevScene& S, v3 o, v3 d, float* tBest, Hit* out,
                                             TraceStats* st)
{
    int stack[kStackSize];
    int sp = 0;
    const int kBlasEnd = (int)0x80000000;
    const int kEmpty = (int)0x80000001;
    int code = S.root;
    bool meshLevel = false;
    int curInst = -1;
    v3 ro = o, rd = d;
    bool fast;
    v3 invd = inv_dir(rd, &fast);
    float m[12];
    uint32_t err = 0;
    const bool cull = S.cullRel >= 0.f;
    float t = *tBest;
    int steps = 0;

    while (true)
    {
        if (++steps > kMaxTraversalSteps) { err |= LF_DEVERR_STEPS; break; }
        if (code == kEmpty)
        {
            if (sp == 0) break;
            code = stack[--sp];
            if (code == kBlasEnd)
            {
                meshLevel = false;
                ro = o;
                rd = d;
                invd = inv_dir(rd, &fast);
                code = kEmpty;
            }
            continue;
        }
        if (code < 0)
        {
            const int payload = ~code;
            if (meshLevel)
            {
                const int first = payload >> 2, cnt = payload & 3;
                if (kStats) { st->leaves++; st->tris += (unsigned)cnt; }
                for (int i = 0; i < cnt; ++i)
                {
                    float u, v;
                    float tt = tri_hit(S.tris + (size_t)(first + i) * 3, ro, rd, &u, &v);
                    if (tt >= 0.f && tt < t)
                    {
                        if (kAny)
                        {
                            *tBest = tt;
                            out->inst = curInst;
                            out->prim = first + i;
                            return err;
                        }
                        t = tt;
                        out->prim = first + i;
                        out->inst = curInst;
                        out->light = -1;
                    }
                }
                code = kEmpty;
            }
            else
            {
                const int inst = payload;
                int root, mat;
                load_instance(S.instances + (size_t)inst * 4, m, &root, &mat);
                if (sp >= kStackCap) { err |= LF_DEVERR_STACK; break; }
                stack[sp++] = kBlasEnd;
                ro = xform(m, o, 1.0f);
                rd = xform(m, d, 0.0f);
                invd = inv_dir(rd, &fast);
                meshLevel = true;
                curInst = inst;
                code = root;
            }
            continue;
        }
        const float4* rec = S.nodes + (size_t)code * 4;
        const float4 f0 = ldg4(rec + 0), f1 = ldg4(rec + 1), f2 = ldg4(rec + 2), f3 = ldg4(rec + 3);
        if (kStats) st->nodes++;
        float eL, eR, hL, hR;
        box_pair(f0, f1, f2, ro, invd, fast, &hL, &hR, &eL, &eR);
        if (cull)
        {
            const float lim = t + t * S.cullRel + S.cullAbs;
            if (eL > lim) hL = -1.0f;
            if (eR > lim) hR = -1.0f;
        }
        const int cL = __float_as_int(f3.x), cR = __float_as_int(f3.y);
        if (hL > 0.f && hR > 0.f)
        {
            int nearC = cL, farC = cR;
            if (hL > hR) { nearC = cR; farC = cL; }
            if (sp >= kStackCap) { err |= LF_DEVERR_STACK; break; }
            stack[sp++] = farC;
            code = nearC;
        }
        else if (hL > 0.f)
            code = cL;
        else if (hR > 0.f)
            code = cR;
        else
            code = kEmpty;
    }
    *tBest = t;
    return err;
}

// ------------------------------------------------------------------ wide traversal
// The 4-wide tree is the reference's binary tree with intermediate levels collapsed: its leaves
// are the reference's leaves and every child box is the box of a reference node. For rays
// whose inverse direction is regular (box_hit_fast), a slab test is monotone in the box, so a
// node's box passes only if every ancestor's box passes: the triangles tested are exactly the
// ones of the leaves whose boxes pass - the reference's set, in a different order. The order
// only matters for hits at the same distance; those are resolved by the reference's
// depth-first order (ref_first). Rays with a degenerate direction take the binary traversal.

// True when the reference's depth-first traversal of the tree holding reference nodes a and b
// reaches a before b: at their lowest common ancestor it descends into the child whose box
// value is smaller (ties left, closest_hit.glsl:172-187), exact box test with the level's ray.
// Arguments are plain values (no reference to the scene) so that calling it leaves the caller's
// registers alone.
static __device__ __noinline__ bool ref_first_at(const int* parent, const float* refNodes, int a, int b, v3 o,
                                                 v3 invd)
{
    int da = 0, db = 0;
    for (int x = a; parent[x] >= 0 && da < 1024; x = parent[x]) ++da;
    for (int x = b; parent[x] >= 0 && db < 1024; x = parent[x]) ++db;
    for (; da > db; --da) a = parent[a];
    for (; db > da; --db) b = parent[b];
    for (int g = 0; g < 1024 && a != b && parent[a] != parent[b]; ++g)
    {
        a = parent[a];
        b = parent[b];
    }
    if (a == b || parent[a] < 0) return false;
    const float* P = refNodes + (size_t)parent[a] * 9;
    const int l = (int)P[6], r = (int)P[7];
    const float* Ln = refNodes + (size_t)l * 9;
    const float* Rn = refNodes + (size_t)r * 9;
    float e;
    const float hL = box_hit(Ln[0], Ln[1], Ln[2], Ln[3], Ln[4], Ln[5], o, invd, &e);
    const float hR = box_hit(Rn[0], Rn[1], Rn[2], Rn[3], Rn[4], Rn[5], o, invd, &e);
    const int nearC = (hL > 0.f && hR > 0.f) ? (hL > hR ? r : l) : (hL > 0.f ? l : r);
    return a == nearC;
}

__device__ __forceinline__ bool ref_first(const DevScene& S, int a, int b, v3 o, v3 invd)
{
    return ref_first_at(S.refParent, S.refNodes, a, b, o, invd);
}

// Binary traversal of one mesh level (the reference's order and exact box test) for an
// object-space ray whose direction is degenerate. Updates t / out like traverse; a hit at the
// same distance as the best hit of another instance is resolved by the instance tree's order
// (world ray wo / winvd, reference nodes of the two instances' leaves).
template <bool kAny>
__device__ __noinline__ uint32_t mesh_binary(const DevScene S, int rootCode, int inst, v3 ro, v3 rd, float* tio,
                                             Hit* out, bool* anyHit, v3 wo, v3 winvd)
{
    int stack[kStackSize];
    int sp = 0;
    const int kEmptyB = (int)0x80000001;
    const v3 invd = 1.0f / rd;
    const bool cull = S.cullRel >= 0.f;
    float t = *tio;
    int code = rootCode;
    uint32_t err = 0;
    for (int steps = 0;; )
    {
        if (++steps > kMaxTraversalSteps) { err |= LF_DEVERR_STEPS; break; }
        if (code == kEmptyB)
        {
            if (sp == 0) break;
            code = stack[--sp];
            continue;
        }
        if (code < 0)
        {
            const int payload = ~code;
            const int first = payload >> 2, cnt = payload & 3;
            for (int i = 0; i < cnt; ++i)
            {
                float u, v;
                const float tt = tri_hit(S.tris + (size_t)(first + i) * 3, ro, rd, &u, &v);
                const bool tie = !kAny && tt == t && tt >= 0.f && out->prim >= 0 && out->inst != inst &&
                                 ref_first(S, S.leafOfInst[inst], S.leafOfInst[out->inst], wo, winvd);
                if ((tt >= 0.f && tt < t) || tie)
                {
                    t = tt;
                    out->prim = first + i;
                    out->inst = inst;
                    out->light = -1;
                    if (kAny)
                    {
                        *anyHit = true;
                        *tio = t;
                        return err;
                    }
                }
            }
            code = kEmptyB;
            continue;
        }
        const float4* rec = S.nodes + (size_t)code * 4;
        const float4 f0 = ldg4(rec + 0), f1 = ldg4(rec + 1), f2 = ldg4(rec + 2), f3 = ldg4(rec + 3);
        float eL, eR;
        float hL = box_hit_exact(f0.x, f0.y, f0.z, f0.w, f1.x, f1.y, ro, invd, &eL);
        float hR = box_hit_exact(f1.z, f1.w, f2.x, f2.y, f2.z, f2.w, ro, invd, &eR);
        if (cull)
        {
            const float lim = t + t * S.cullRel + S.cullAbs;
            if (eL > lim) hL = -1.0f;
            if (eR > lim) hR = -1.0f;
        }
        const int cL = __float_as_int(f3.x), cR = __float_as_int(f3.y);
        if (hL > 0.f && hR > 0.f)
        {
            int nearC = cL, farC = cR;
            if (hL > hR) { nearC = cR; farC = cL; }
            if (sp >= kStackCap) { err |= LF_DEVERR_STACK; break; }
            stack[sp++] = farC;
            code = nearC;
        }
        else if (hL > 0.f)
            code = cL;
        else if (hR > 0.f)
            code = cR;
        else
            code = kEmptyB;
    }
    *tio = t;
    return err;
}

// Two floats in one 64-bit register pair, for the packed f32x2 operations of sm_100 and later:
// sub.rn.f32x2 / mul.rn.f32x2 round each lane exactly as sub.rn.f32 / mul.rn.f32 do.
typedef unsigned long long f2_t;

__device__ __forceinline__ f2_t f2_dup(float a)
{
    f2_t r;
    asm("mov.b64 %0, {%1, %1};" : "=l"(r) : "f"(a));
    return r;
}

__device__ __forceinline__ f2_t f2_sub(f2_t a, f2_t b)
{
    f2_t r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b)
{
    f2_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

__device__ __forceinline__ void f2_split(f2_t v, float& a, float& b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}

// Slab distances of the kWide children of a wide node (box_hit_fast's t0 and t1 for each),
// for a ray whose inverse direction is finite and non-zero: (bound - o) * invd for two children
// per packed instruction. On an axis with invd > 0 the lower bound's distance is the smaller of
// the two (lo <= hi, and subtracting o and multiplying by a positive number keep the order), on
// an axis with invd < 0 the upper bound's: the bounds are read in near / far order for the
// ray's octant, and box_hit_fast's per-axis min / max reduce to t0 = max(near) and
// t1 = min(far) with the same values. An unused slot's empty box (lo = +inf, hi = -inf) gives
// t0 = +inf and t1 = -inf for every such ray: (+inf - o) * invd and (-inf - o) * invd are
// +inf and -inf in near / far order whatever the sign of invd.
__device__ __forceinline__ void wide_slabs(const float4* rec, v3 ro, v3 invd, float t0[kWide], float t1[kWide])
{
    constexpr int G = kWide / 4;   // float4 per group
    const f2_t ro2[3] = {f2_dup(ro.x), f2_dup(ro.y), f2_dup(ro.z)};
    const f2_t iv2[3] = {f2_dup(invd.x), f2_dup(invd.y), f2_dup(invd.z)};
    const int neg[3] = {invd.x < 0.f ? 1 : 0, invd.y < 0.f ? 1 : 0, invd.z < 0.f ? 1 : 0};
    ulonglong2 nearB[3][G], farB[3][G];   // per axis the near and far bounds, two children per 64 bits
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int h4 = 0; h4 < G; ++h4)
        {
            nearB[a][h4] = __ldg(reinterpret_cast<const ulonglong2*>(rec + (2 * a + neg[a]) * G + h4));
            farB[a][h4] = __ldg(reinterpret_cast<const ulonglong2*>(rec + (2 * a + 1 - neg[a]) * G + h4));
        }
#pragma unroll
    for (int h4 = 0; h4 < G; ++h4)
#pragma unroll
        for (int half = 0; half < 2; ++half)
        {
            float n[3][2], f[3][2];
#pragma unroll
            for (int a = 0; a < 3; ++a)
            {
                const f2_t lo = half ? nearB[a][h4].y : nearB[a][h4].x;
                const f2_t hi = half ? farB[a][h4].y : farB[a][h4].x;
                f2_split(f2_mul(f2_sub(lo, ro2[a]), iv2[a]), n[a][0], n[a][1]);
                f2_split(f2_mul(f2_sub(hi, ro2[a]), iv2[a]), f[a][0], f[a][1]);
            }
#pragma unroll
            for (int c = 0; c < 2; ++c)
            {
                const int j = h4 * 4 + half * 2 + c;
                t1[j] = fmin3_hw(f[0][c], f[1][c], f[2][c]);
                t0[j] = fmax3_hw(n[0][c], n[1][c], n[2][c]);
            }
        }
}

// Compare-exchange of two (key, child code) pairs by key: the codes travel with their keys, so
// no per-slot lookup is needed after the sort.
__device__ __forceinline__ void sort2(uint32_t& a, uint32_t& b, int& ca, int& cb)
{
    const bool swap = b < a;
    const uint32_t lo = swap ? b : a, hi = swap ? a : b;
    const int clo = swap ? cb : ca, chi = swap ? ca : cb;
    a = lo;
    b = hi;
    ca = clo;
    cb = chi;
}

// Child hits of one wide node, nearest entry first: hc[0..nh). The children are ordered by a
// sorting network on keys that hold the entry distance's bits (entries are >= 0, so their bit
// patterns order like the values) with the child slot in the low bits; children whose entries
// differ only in those bits are ordered by slot. The visiting order only decides how early the
// closest hit is found, not which hit is returned.
__device__ __forceinline__ int wide_node(const DevScene& S, int code, v3 ro, v3 invd, float lim, int* hc)
{
    const float4* rec = S.wnodes + (size_t)code * kWideF4;
    constexpr int G = kWide / 4;   // float4 per group
    constexpr uint32_t kSlotMask = kWide - 1;
    float t0[kWide], t1[kWide];
    wide_slabs(rec, ro, invd, t0, t1);
    uint32_t key[kWide];
    int child[kWide];
#pragma unroll
    for (int h4 = 0; h4 < G; ++h4)
    {
        const int4 c = __ldg(reinterpret_cast<const int4*>(rec + 6 * G + h4));
        child[h4 * 4 + 0] = c.x;
        child[h4 * 4 + 1] = c.y;
        child[h4 * 4 + 2] = c.z;
        child[h4 * 4 + 3] = c.w;
    }
    int nh = 0;
#pragma unroll
    for (int j = 0; j < kWide; ++j)
    {
        // box_hit_fast's value is > 0 exactly when t1 >= t0 and t1 > 0, and the entry
        // max(t0, 0) must not exceed lim (> 0). With e = max(t0, smallest positive float) the
        // three tests are one, e <= min(t1, lim): for t0 > 0, e = t0; for t0 <= 0 it asks
        // t1 > 0 (lim > 0 always). e's bits differ from max(t0, 0)'s only below the key's slot
        // bits. An unused slot (t0 = +inf, t1 = -inf) fails.
        const float e = fmaxf(t0[j], 1.401298464e-45f);
        const bool hit = e <= fminf(t1[j], lim);
        key[j] = hit ? ((__float_as_uint(e) & ~kSlotMask) | (uint32_t)j) : 0xFFFFFFFFu;
        nh += hit ? 1 : 0;
    }
#define LF_S2(a, b) sort2(key[a], key[b], child[a], child[b])
    if constexpr (kWide == 4)
    {
        LF_S2(0, 1);
        LF_S2(2, 3);
        LF_S2(0, 2);
        LF_S2(1, 3);
        LF_S2(1, 2);
    }
    else
    {
        // Batcher's odd-even merge sort of 8
#pragma unroll
        for (int a = 0; a < 8; a += 2) LF_S2(a, a + 1);
        LF_S2(0, 2); LF_S2(1, 3); LF_S2(4, 6); LF_S2(5, 7);
        LF_S2(1, 2); LF_S2(5, 6);
        LF_S2(0, 4); LF_S2(1, 5); LF_S2(2, 6); LF_S2(3, 7);
        LF_S2(2, 4); LF_S2(3, 5);
        LF_S2(1, 2); LF_S2(3, 4); LF_S2(5, 6);
    }
#undef LF_S2
#pragma unroll
    for (int k = 0; k < kWide; ++k) hc[k] = child[k];
    return nh;
}

constexpr int kWideBlasEnd = (int)0x80000000;   // stack marker: leave the instance
constexpr int kWideNone = (int)0x80000001;      // no next node

// Occlusion form of wide_node: any-hit returns a boolean, so the order in which the children
// are visited cannot change its answer (AnyHit, anyhit.glsl:7-173, accepts the first triangle
// with t < maxDist it meets). The hit children are taken in slot order without keys or a
// sorting network: the first is returned (kWideNone if none), the others are pushed. Returns
// kWideEmpty, pushing nothing, when the pushes would overflow the stack.
__device__ __forceinline__ int wide_node_any(const DevScene& S, int code, v3 ro, v3 invd, float lim, int* stack,
                                             int& sp)
{
    const float4* rec = S.wnodes + (size_t)code * kWideF4;
    constexpr int G = kWide / 4;
    float t0[kWide], t1[kWide];
    wide_slabs(rec, ro, invd, t0, t1);
    bool hit[kWide];
    int nh = 0;
#pragma unroll
    for (int j = 0; j < kWide; ++j)
    {
        hit[j] = fmaxf(t0[j], 1.401298464e-45f) <= fminf(t1[j], lim);   // as in wide_node
        nh += hit[j] ? 1 : 0;
    }
    if (sp + nh - 1 > kWideStack) return kWideEmpty;
    int child[kWide];
#pragma unroll
    for (int h4 = 0; h4 < G; ++h4)
    {
        const int4 c = __ldg(reinterpret_cast<const int4*>(rec + 6 * G + h4));
        child[h4 * 4 + 0] = c.x;
        child[h4 * 4 + 1] = c.y;
        child[h4 * 4 + 2] = c.z;
        child[h4 * 4 + 3] = c.w;
    }
    int next = kWideNone;
#pragma unroll
    for (int j = 0; j < kWide; ++j)
        if (hit[j])
        {
            if (next != kWideNone) stack[sp++] = next;
            next = child[j];
        }
    return next;
}

// Two-level traversal of the wide tree as a state machine: wide_step visits one node or leaf
// and folds the stack pop into the same step. Leaves are triangle runs on the mesh level and
// instances on the instance level; entering an instance pushes a marker and switches to the
// object-space ray. Equal-distance hits are ordered by the reference's own visiting order
// (ref_first). The state lives in registers (the stack in local memory), so a persistent
// kernel can interleave rays without saving it.
struct WideRay
{
    v3 o, d, winvd;    // world-space ray
    v3 ro, rd, invd;   // ray of the current level
    float t;           // current end of the ray (best hit distance)
    int code;          // next node: >= 0 inner record, < 0 leaf, kWideNone none
    int sp, curInst, steps;
    bool meshLevel;
    uint32_t err;
};


// Starts a traversal of a ray with a regular inverse direction (inv_dir's `fast`).
__device__ __forceinline__ void wide_init(const DevScene& S, WideRay& w, v3 o, v3 d, v3 winvd, float tmax)
{
    w.o = o;
    w.d = d;
    w.winvd = winvd;
    w.ro = o;
    w.rd = d;
    w.invd = winvd;
    w.t = tmax;
    w.code = S.wroot;
    w.sp = 0;
    w.curInst = -1;
    w.steps = 0;
    w.meshLevel = false;
    w.err = 0;
}

// One traversal step; returns true when the traversal has ended (w.t and `out` hold the result).
template <bool kAny>
__device__ __forceinline__ bool wide_step(const DevScene& S, WideRay& w, int* stack, Hit& out)
{
    if (++w.steps > kMaxTraversalSteps)
    {
        w.err |= LF_DEVERR_STEPS;
        return true;
    }
    int code = w.code;
    if (kAny && code >= 0)
    {
        const float lim = S.cullRel >= 0.f ? w.t + w.t * S.cullRel + S.cullAbs : 3.4e38f;
        code = wide_node_any(S, code, w.ro, w.invd, lim, stack, w.sp);
        if (code == kWideEmpty)
        {
            w.err |= LF_DEVERR_STACK;
            return true;
        }
    }
    else if (code >= 0)
    {
        int hc[kWide];
        const float lim = S.cullRel >= 0.f ? w.t + w.t * S.cullRel + S.cullAbs : 3.4e38f;
        const int nh = wide_node(S, code, w.ro, w.invd, lim, hc);
        if (w.sp + nh - 1 > kWideStack)
        {
            w.err |= LF_DEVERR_STACK;
            return true;
        }
#pragma unroll
        for (int k = kWide - 1; k >= 1; --k)
            if (k < nh) stack[w.sp++] = hc[k];
        code = nh > 0 ? hc[0] : kWideNone;
    }
    else if (w.meshLevel)
    {
        const int payload = ~code;
        const int first = payload >> 2, cnt = payload & 3;
        code = kWideNone;
        for (int i = 0; i < cnt; ++i)
        {
            const int prim = first + i;
            const float tt = tri_hit_upto(S.tris + (size_t)prim * 3, w.ro, w.rd, w.t);
            if (tt >= 0.f)
            {
                bool take = tt < w.t;
                if (!take && !kAny && out.prim >= 0)
                {
                    // equal distance: the reference keeps the one it reaches first
                    if (w.curInst == out.inst)
                    {
                        const int la = S.leafOfTri[prim], lb = S.leafOfTri[out.prim];
                        take = la == lb ? prim < out.prim : ref_first(S, la, lb, w.ro, w.invd);
                    }
                    else
                        take = ref_first(S, S.leafOfInst[w.curInst], S.leafOfInst[out.inst], w.o, w.winvd);
                }
                if (take)
                {
                    w.t = tt;
                    out.prim = prim;
                    out.inst = w.curInst;
                    out.light = -1;
                    if (kAny) return true;
                }
            }
        }
    }
    else
    {
        const int inst = ~code;
        const float4* ir = S.instances + (size_t)inst * 4;
        float m[12];
        int root, mat;
        load_instance(ir, m, &root, &mat);
        const float4 e3 = ldg4(ir + 3);
        const v3 iro = xform(m, w.o, 1.0f), ird = xform(m, w.d, 0.0f);
        bool ofast;
        const v3 iinvd = inv_dir(ird, &ofast);
        code = kWideNone;
        if (!ofast)
        {
            // copies, so that the state keeps no address and stays in registers
            bool anyHit = false;
            float tm = w.t;
            Hit hm = out;
            w.err |= mesh_binary<kAny>(S, root, inst, iro, ird, &tm, &hm, &anyHit, w.o, w.winvd);
            w.t = tm;
            out = hm;
            if (kAny && anyHit) return true;
        }
        else
        {
            if (w.sp >= kWideStack)
            {
                w.err |= LF_DEVERR_STACK;
                return true;
            }
            stack[w.sp++] = kWideBlasEnd;
            w.ro = iro;
            w.rd = ird;
            w.invd = iinvd;
            w.meshLevel = true;
            w.curInst = inst;
            code = __float_as_int(e3.z);
        }
    }
    if (code == kWideNone)
    {
        if (w.sp == 0) return true;
        code = stack[--w.sp];
        if (code == kWideBlasEnd)
        {
            // leave the instance; the entry below the marker is an instance-level one
            w.meshLevel = false;
            w.ro = w.o;
            w.rd = w.d;
            w.invd = w.winvd;
            if (w.sp == 0) return true;
            code = stack[--w.sp];
        }
    }
    w.code = code;
    return false;
}

template <bool kAny>
__device__ __forceinline__ uint32_t traverse_wide(const DevScene& S, v3 o, v3 d, float* tBest, Hit* out)
{
    bool fast;
    const v3 winvd = inv_dir(d, &fast);
    if (!fast) return traverse<kAny, false>(S, o, d, tBest, out, nullptr);
    WideRay w;
    int stack[kWideStack];
    wide_init(S, w, o, d, winvd, *tBest);
    Hit h = *out;
    while (!wide_step<kAny>(S, w, stack, h)) {}
    *out = h;
    *tBest = w.t;
    return w.err;
}

// Closest hit: analytic lights first (closest_hit.glsl:13-67), then the BVH.
template <bool kStats>
__device__ __forceinline__ uint32_t closest_hit(const DevScene& S, v3 o, v3 d, float tInit, bool useLights,
                                                Hit* out, TraceStats* st)
{
    float t = tInit;
    out->inst = -1;
    out->prim = -1;
    out->light = -1;
    if (useLights)
    {
        for (int i = 0; i < S.numLights; ++i)
        {
            const DevLight& L = S.lights[i];
            float dd;
            if (L.type == 0.f)
            {
                v3 n(L.normal[0], L.normal[1], L.normal[2]);
                if (lfc::dot(n, d) > 0.f) continue;
                dd = rect_intersect(L, o, d);
                if (dd < 0.f) dd = kInfinity;
                if (dd < t) { t = dd; out->light = i; }
            }
            if (L.type == 1.f)
            {
                dd = sphere_intersect(L, o, d);
                if (dd < 0.f) dd = kInfinity;
                if (dd < t) { t = dd; out->light = i; }
            }
        }
    }
    uint32_t err = (!kStats && S.wnodes && S.wideOn) ? traverse_wide<false>(S, o, d, &t, out)
                                                      : traverse<false, kStats>(S, o, d, &t, out, st);
    out->t = t;
    return err;
}

// Occlusion: lights (two-sided quads, anyhit.glsl:15-50), then the BVH.
template <bool kStats>
__device__ __forceinline__ uint32_t any_hit(const DevScene& S, v3 o, v3 d, float maxDist, bool useLights,
                                            bool* occluded, Hit* out, TraceStats* st)
{
    out->inst = -1;
    out->prim = -1;
    out->light = -1;
    *occluded = false;
    if (useLights)
    {
        for (int i = 0; i < S.numLights; ++i)
        {
            const DevLight& L = S.lights[i];
            if (L.type == 0.f)
            {
                float dd = rect_intersect(L, o, d);
                if (dd > 0.f && dd < maxDist) { *occluded = true; out->light = i; out->t = dd; return 0; }
            }
            if (L.type == 1.f)
            {
                float dd = sphere_intersect(L, o, d);
                if (dd > 0.f && dd < maxDist) { *occluded = true; out->light = i; out->t = dd; return 0; }
            }
        }
    }
    float t = maxDist;
    uint32_t err = (!kStats && S.wnodes && S.wideOn) ? traverse_wide<true>(S, o, d, &t, out)
                                                     : traverse<true, kStats>(S, o, d, &t, out, st);
    *occluded = out->prim >= 0;
    out->t = *occluded ? t : kInfinity;
    return err;
}
}

namespace lfd
{
// Resumable form of `traverse` for persistent kernels: the same state machine and visit
// order, run for a bounded number of iterations per call so that a warp can refill
// finished lanes with new rays between calls.
struct TravState
{
    v3 o, d, ro, rd, invd;
    float t;
    int code;
    int sp;
    int curInst;
    int hitInst, hitPrim;
    int steps;
    uint32_t err;
    bool meshLevel;
    bool fast;
    int stack[kStackSize];
};

constexpr int kTravBlasEnd = (int)0x80000000;
constexpr int kTravEmpty = (int)0x80000001;

__device__ __forceinline__ void trav_init(TravState& s, const DevScene& S, v3 o, v3 d, float t)
{
    s.o = o;
    s.d = d;
    s.ro = o;
    s.rd = d;
    s.invd = inv_dir(d, &s.fast);
    s.t = t;
    s.code = S.root;
    s.sp = 0;
    s.curInst = -1;
    s.hitInst = -1;
    s.hitPrim = -1;
    s.steps = 0;
    s.err = 0;
    s.meshLevel = false;
}

// Returns true when the traversal has finished (or an error ended it).
template <bool kAny>
__device__ __forceinline__ bool trav_run(TravState& s, const DevScene& S, int budget)
{
    const bool cull = S.cullRel >= 0.f;
    for (int it = 0; it < budget; ++it)
    {
        if (++s.steps > kMaxTraversalSteps)
        {
            s.err |= LF_DEVERR_STEPS;
            return true;
        }
        int code = s.code;
        if (code == kTravEmpty)
        {
            if (s.sp == 0) return true;
            code = s.stack[--s.sp];
            if (code == kTravBlasEnd)
            {
                s.meshLevel = false;
                s.ro = s.o;
                s.rd = s.d;
                s.invd = inv_dir(s.d, &s.fast);
                code = kTravEmpty;
            }
            s.code = code;
            continue;
        }
        if (code < 0)
        {
            const int payload = ~code;
            if (s.meshLevel)
            {
                const int first = payload >> 2, cnt = payload & 3;
                for (int i = 0; i < cnt; ++i)
                {
                    float u, v;
                    float tt = tri_hit(S.tris + (size_t)(first + i) * 3, s.ro, s.rd, &u, &v);
                    if (tt >= 0.f && tt < s.t)
                    {
                        s.t = tt;
                        s.hitPrim = first + i;
                        s.hitInst = s.curInst;
                        if (kAny) return true;
                    }
                }
                s.code = kTravEmpty;
            }
            else
            {
                float m[12];
                int root, mat;
                load_instance(S.instances + (size_t)payload * 4, m, &root, &mat);
                if (s.sp >= kStackCap)
                {
                    s.err |= LF_DEVERR_STACK;
                    return true;
                }
                s.stack[s.sp++] = kTravBlasEnd;
                s.ro = xform(m, s.o, 1.0f);
                s.rd = xform(m, s.d, 0.0f);
                s.invd = inv_dir(s.rd, &s.fast);
                s.meshLevel = true;
                s.curInst = payload;
                s.code = root;
            }
            continue;
        }
        const float4* rec = S.nodes + (size_t)code * 4;
        const float4 f0 = ldg4(rec + 0), f1 = ldg4(rec + 1), f2 = ldg4(rec + 2), f3 = ldg4(rec + 3);
        float eL, eR, hL, hR;
        box_pair(f0, f1, f2, s.ro, s.invd, s.fast, &hL, &hR, &eL, &eR);
        if (cull)
        {
            const float lim = s.t + s.t * S.cullRel + S.cullAbs;
            if (eL > lim) hL = -1.0f;
            if (eR > lim) hR = -1.0f;
        }
        const int cL = __float_as_int(f3.x), cR = __float_as_int(f3.y);
        if (hL > 0.f && hR > 0.f)
        {
            int nearC = cL, farC = cR;
            if (hL > hR)
            {
                nearC = cR;
                farC = cL;
            }
            if (s.sp >= kStackCap)
            {
                s.err |= LF_DEVERR_STACK;
                return true;
            }
            s.stack[s.sp++] = farC;
            s.code = nearC;
        }
        else if (hL > 0.f)
            s.code = cL;
        else if (hR > 0.f)
            s.code = cR;
        else
            s.code = kTravEmpty;
    }
    return false;
}

// Analytic lights of ClosestHit (closest_hit.glsl:13-67): returns the initial t and the
// light index (or -1).
__device__ __forceinline__ float lights_closest(const DevScene& S, v3 o, v3 d, float t, int* light)
{
    *light = -1;
    for (int i = 0; i < S.numLights; ++i)
    {
        const DevLight& L = S.lights[i];
        float dd;
        if (L.type == 0.f)
        {
            v3 n(L.normal[0], L.normal[1], L.normal[2]);
            if (lfc::dot(n, d) > 0.f) continue;
            dd = rect_intersect(L, o, d);
            if (dd < 0.f) dd = kInfinity;
            if (dd < t) { t = dd; *light = i; }
        }
        if (L.type == 1.f)
        {
            dd = sphere_intersect(L, o, d);
            if (dd < 0.f) dd = kInfinity;
            if (dd < t) { t = dd; *light = i; }
        }
    }
    return t;
}

// Analytic lights of AnyHit (anyhit.glsl:15-50).
__device__ __forceinline__ bool lights_any(const DevScene& S, v3 o, v3 d, float maxDist)
{
    for (int i = 0; i < S.numLights; ++i)
    {
        const DevLight& L = S.lights[i];
        if (L.type == 0.f)
        {
            float dd = rect_intersect(L, o, d);
            if (dd > 0.f && dd < maxDist) return true;
        }
        if (L.type == 1.f)
        {
            float dd = sphere_intersect(L, o, d);
            if (dd > 0.f && dd < maxDist) return true;
        }
    }
    return false;
}
}
