// Oracle: scalar C++ restatement of the reference path tracer (shaders/renderer.glsl and
// shaders/common/{globals,intersection,closest_hit,anyhit,sampling,disney,pathtrace}.glsl),
// run multithreaded on the host. TEST INFRASTRUCTURE ONLY: tests, the smoke check and the
// bench's CPU baseline load it to check results; the product never links or calls it.
//
// It reads the scene in the reference's own flat layouts (36-byte nodes with float-encoded
// indices, int3 triangle indices, float4 vertices/normals, 112-byte materials, 64-byte
// transforms, 60-byte lights) and follows the GLSL line by line: the two-level traversal
// with its stack[64] and sentinels, texelFetch-style lookups, the light loop, the Disney
// lobes and the bounce loop, with one rand() call per call in the shader.
// Operations GLSL leaves implementation-defined (transcendentals, inverse(), texture
// filtering) use the project's arithmetic contract (csrc/lf_contract.h, csrc/lf_vec.h);
// texture lookups are restated here from that definition.
// Pinning: the BVH/scene arrays it consumes are checked byte-for-byte against the
// reference host code compiled from source, and its radiance against the reference shader
// source compiled for the CPU (golden vectors in tests/golden/).
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "lf_vec.h"

using lfc::v2;
using lfc::v3;

namespace
{
const float PI = 3.14159265358979323f;
const float TWO_PI = 6.28318530717958648f;
const float INF_T = 1000000.0f;
const float EPS = 0.001f;

struct View
{
    const float* nodes;
    int num_nodes, top;
    const int* vidx;
    int num_tris;
    const float* verts;
    const float* norms;
    int num_vertices;
    const float* mats;
    int num_materials;
    const float* xf;
    int num_instances;
    const float* lights;
    int num_lights;
    const float* env_rgb;
    const float* env_marg;
    const float* env_cond;
    int env_w, env_h;
    const uint8_t* tex;
    int tex_w, tex_h, num_tex;
};

struct Options
{
    int lights;        // LIGHTS
    float cullRel;     // < 0: no culling (the reference)
    float cullAbs;
};

struct Prepared
{
    View v;
    std::vector<float> inv;   // 16 per instance, GLSL inverse()
    std::vector<float> nrm;   // 9 per instance, transpose(inverse(mat3(M)))
};

struct Counters
{
    uint64_t nodes = 0, tris = 0, leaves = 0, overflow = 0, instances = 0;
};

// ------------------------------------------------------------------ texel fetches
inline v3 node_v(const View& V, int index, int texel)
{
    const float* p = V.nodes + (size_t)index * 9 + texel * 3;
    return v3(p[0], p[1], p[2]);
}

inline v3 vec3_of(const float* p) { return v3(p[0], p[1], p[2]); }

struct LightData
{
    v3 position, emission, u, v;
    float radius, area, type;
};

inline LightData light_fetch(const View& V, int i)
{
    const float* p = V.lights + (size_t)i * 15;
    return LightData{vec3_of(p), vec3_of(p + 3), vec3_of(p + 6), vec3_of(p + 9), p[12], p[13], p[14]};
}

// ------------------------------------------------------------------ intersection.glsl
float SphereIntersect(float rad, v3 pos, v3 ro, v3 rd)
{
    v3 op = pos - ro;
    float eps = 0.001f;
    float b = lfc::dot(op, rd);
    float det = b * b - lfc::dot(op, op) + rad * rad;
    if (det < 0.0f) return INF_T;
    det = sqrtf(det);
    float t1 = b - det;
    if (t1 > eps) return t1;
    float t2 = b + det;
    if (t2 > eps) return t2;
    return INF_T;
}

float RectIntersect(v3 pos, v3 u, v3 v, v3 n, float planeW, v3 ro, v3 rd)
{
    float dt = lfc::dot(rd, n);
    float t = (planeW - lfc::dot(n, ro)) / dt;
    if (t > EPS)
    {
        v3 p = ro + rd * t;
        v3 vi = p - pos;
        float a1 = lfc::dot(u, vi);
        if (a1 >= 0.f && a1 <= 1.f)
        {
            float a2 = lfc::dot(v, vi);
            if (a2 >= 0.f && a2 <= 1.f) return t;
        }
    }
    return INF_T;
}

// returns the GLSL value and the entry distance max(t0, 0) used by the optional cull; rays
// with a zero, denormal or non-finite inverse direction component are never culled (their slab
// values can be NaN or infinite, and the entry is then no lower bound of the hit distance)
inline bool finite_nonzero(float x) { return std::fabs(x) < 3.0e38f && x != 0.f; }

float AABBIntersect(v3 mn, v3 mx, v3 ro, v3 rd, float* entry)
{
    v3 invdir = 1.0f / rd;
    v3 f = (mx - ro) * invdir;
    v3 n = (mn - ro) * invdir;
    v3 tmax = lfc::vmax(f, n);
    v3 tmin = lfc::vmin(f, n);
    float t1 = lfc::fmin_g(tmax.x, lfc::fmin_g(tmax.y, tmax.z));
    float t0 = lfc::fmax_g(tmin.x, lfc::fmax_g(tmin.y, tmin.z));
    const bool regular = finite_nonzero(invdir.x) && finite_nonzero(invdir.y) && finite_nonzero(invdir.z);
    *entry = regular && t0 > 0.f ? t0 : 0.f;
    return (t1 >= t0) ? (t0 > 0.f ? t0 : t1) : -1.0f;
}

// vec3(M * vec4(p, w)) with M given column-major (GLSL order)
inline v3 mul4(const float* m, v3 p, float w) { return lfc::mul4_point(m, p, w); }

struct HitRec
{
    float t;
    bool isEmitter;
    int light;
    int triPacked;
    int inst;
    int matID;
    v3 bary;
    v3 fhp;
    v3 tempTex;
    float tieT = -1.0f;   // distance of the last candidate rejected for t == tBest (test diagnostics only)
};

// Two-level traversal shared by ClosestHit (closest_hit.glsl:69-201) and AnyHit
// (anyhit.glsl:252-374); `any` returns at the first accepted triangle.
bool Traverse(const Prepared& P, const Options& O, v3 ro0, v3 rd0, float& t, bool any, HitRec* h, Counters& c)
{
    const View& V = P.v;
    int stack[64];
    int ptr = 0;
    stack[ptr++] = -1;
    int idx = V.top;
    int currMatID = 0;
    int currInst = -1;
    bool meshBVH = false;
    v3 r_o = ro0, r_d = rd0;
    const float* inv = nullptr;
    const bool cull = O.cullRel >= 0.f;

    while (idx > -1 || meshBVH)
    {
        int n = idx;
        if (meshBVH && idx < 0)
        {
            meshBVH = false;
            idx = stack[--ptr];
            r_o = ro0;
            r_d = rd0;
            continue;
        }
        v3 lr = node_v(V, n, 2);
        int leftIndex = (int)lr.x, rightIndex = (int)lr.y, leaf = (int)lr.z;
        if (leaf > 0)
        {
            c.leaves++;
            for (int i = 0; i < rightIndex; i++)
            {
                int index = leftIndex + i;
                const int* vi = V.vidx + (size_t)index * 3;
                const float* v0 = V.verts + (size_t)vi[0] * 4;
                const float* v1 = V.verts + (size_t)vi[1] * 4;
                const float* v2p = V.verts + (size_t)vi[2] * 4;
                c.tris++;
                v3 e0 = vec3_of(v1) - vec3_of(v0);
                v3 e1 = vec3_of(v2p) - vec3_of(v0);
                v3 pv = lfc::cross(r_d, e1);
                float det = lfc::dot(e0, pv);
                v3 tv = r_o - vec3_of(v0);
                v3 qv = lfc::cross(tv, e0);
                float ux = lfc::dot(tv, pv) / det;
                float uy = lfc::dot(r_d, qv) / det;
                float uz = lfc::dot(e1, qv) / det;
                float uw = 1.0f - ux - uy;
                const bool inside = ux >= 0.f && uy >= 0.f && uz >= 0.f && uw >= 0.f;
                if (!any && inside && uz == t) h->tieT = uz;   // equal-distance competitor (strict < keeps the first)
                if (inside && uz < t)
                {
                    if (any)
                    {
                        t = uz;
                        if (h) { h->triPacked = index; h->inst = currInst; }
                        return true;
                    }
                    t = uz;
                    h->isEmitter = false;
                    h->light = -1;
                    h->triPacked = index;
                    h->inst = currInst;
                    h->matID = currMatID;
                    h->bary = v3(uw, ux, uy);
                    h->tempTex = v3(v0[3], v1[3], v2p[3]);
                    v3 fhp = r_o + r_d * t;
                    const float* M = V.xf + (size_t)currInst * 16;
                    h->fhp = mul4(M, fhp, 1.0f);
                }
            }
        }
        else if (leaf < 0)
        {
            c.instances++;
            idx = leftIndex;
            int inst = -leaf - 1;
            inv = &P.inv[(size_t)inst * 16];
            r_o = mul4(inv, ro0, 1.0f);
            r_d = mul4(inv, rd0, 0.0f);
            if (ptr >= 64) { c.overflow++; break; }
            stack[ptr++] = -1;
            meshBVH = true;
            currMatID = rightIndex;
            currInst = inst;
            continue;
        }
        else
        {
            c.nodes++;
            float eL, eR;
            float leftHit = AABBIntersect(node_v(V, leftIndex, 0), node_v(V, leftIndex, 1), r_o, r_d, &eL);
            float rightHit = AABBIntersect(node_v(V, rightIndex, 0), node_v(V, rightIndex, 1), r_o, r_d, &eR);
            if (cull)
            {
                float lim = t + t * O.cullRel + O.cullAbs;
                if (eL > lim) leftHit = -1.0f;
                if (eR > lim) rightHit = -1.0f;
            }
            if (leftHit > 0.0f && rightHit > 0.0f)
            {
                int deferred;
                if (leftHit > rightHit)
                {
                    idx = rightIndex;
                    deferred = leftIndex;
                }
                else
                {
                    idx = leftIndex;
                    deferred = rightIndex;
                }
                if (ptr >= 64) { c.overflow++; break; }
                stack[ptr++] = deferred;
                continue;
            }
            else if (leftHit > 0.f)
            {
                idx = leftIndex;
                continue;
            }
            else if (rightHit > 0.f)
            {
                idx = rightIndex;
                continue;
            }
        }
        idx = stack[--ptr];
    }
    return false;
}

// ClosestHit (closest_hit.glsl:7-205): returns t; the hit record keeps stale fields when
// nothing closer than an analytic light is found, exactly like the shader's State.
float ClosestHit(const Prepared& P, const Options& O, v3 ro, v3 rd, HitRec& st, float& lightPdf, v3& lightEmission,
                 Counters& c, float tInit = INF_T)
{
    const View& V = P.v;
    float t = tInit;
    if (O.lights)
    {
        for (int i = 0; i < V.num_lights; i++)
        {
            LightData L = light_fetch(V, i);
            float d;
            if (L.type == 0.f)
            {
                v3 normal = lfc::normalize(lfc::cross(L.u, L.v));
                if (lfc::dot(normal, rd) > 0.f) continue;
                float planeW = lfc::dot(normal, L.position);
                v3 u = L.u * (1.0f / lfc::dot(L.u, L.u));
                v3 v = L.v * (1.0f / lfc::dot(L.v, L.v));
                d = RectIntersect(L.position, u, v, normal, planeW, ro, rd);
                if (d < 0.f) d = INF_T;
                if (d < t)
                {
                    t = d;
                    float cosTheta = lfc::dot(-rd, normal);
                    lightPdf = (t * t) / (L.area * cosTheta);
                    lightEmission = L.emission;
                    st.isEmitter = true;
                    st.light = i;
                }
            }
            if (L.type == 1.f)
            {
                d = SphereIntersect(L.radius, L.position, ro, rd);
                if (d < 0.f) d = INF_T;
                if (d < t)
                {
                    t = d;
                    lightPdf = (t * t) / L.area;
                    lightEmission = L.emission;
                    st.isEmitter = true;
                    st.light = i;
                }
            }
        }
    }
    Traverse(P, O, ro, rd, t, false, &st, c);
    st.t = t;
    return t;
}

bool AnyHit(const Prepared& P, const Options& O, v3 ro, v3 rd, float maxDist, Counters& c)
{
    const View& V = P.v;
    if (O.lights)
    {
        for (int i = 0; i < V.num_lights; i++)
        {
            LightData L = light_fetch(V, i);
            if (L.type == 0.f)
            {
                v3 normal = lfc::normalize(lfc::cross(L.u, L.v));
                float planeW = lfc::dot(normal, L.position);
                v3 u = L.u * (1.0f / lfc::dot(L.u, L.u));
                v3 v = L.v * (1.0f / lfc::dot(L.v, L.v));
                float d = RectIntersect(L.position, u, v, normal, planeW, ro, rd);
                if (d > 0.0f && d < maxDist) return true;
            }
            if (L.type == 1.f)
            {
                float d = SphereIntersect(L.radius, L.position, ro, rd);
                if (d > 0.0f && d < maxDist) return true;
            }
        }
    }
    float t = maxDist;
    return Traverse(P, O, ro, rd, t, true, nullptr, c);
}

// ------------------------------------------------------------------ textures (GL semantics
// as fixed by the contract: REPEAT wrap, nearest = floor(u*size), linear with texel centres
// at +0.5, weights combined as ((T00(1-a) + T10 a)(1-b) + (T01(1-a) + T11 a) b)).
int wrapi(int i, int n)
{
    int r = i % n;
    return r < 0 ? r + n : r;
}

void tex_nearest2(const float* t, int w, int h, float u, float v, float out[2])
{
    int x = wrapi((int)floorf(u * (float)w), w);
    int y = wrapi((int)floorf(v * (float)h), h);
    out[0] = t[((size_t)y * w + x) * 2 + 0];
    out[1] = t[((size_t)y * w + x) * 2 + 1];
}

v3 tex_linear3(const float* t, int w, int h, float u, float v)
{
    float xf = u * (float)w - 0.5f, yf = v * (float)h - 0.5f;
    float x0f = floorf(xf), y0f = floorf(yf);
    float a = xf - x0f, b = yf - y0f;
    int x0 = wrapi((int)x0f, w), x1 = wrapi((int)x0f + 1, w), y0 = wrapi((int)y0f, h), y1 = wrapi((int)y0f + 1, h);
    float r[3];
    for (int k = 0; k < 3; ++k)
    {
        float t00 = t[((size_t)y0 * w + x0) * 3 + k], t10 = t[((size_t)y0 * w + x1) * 3 + k];
        float t01 = t[((size_t)y1 * w + x0) * 3 + k], t11 = t[((size_t)y1 * w + x1) * 3 + k];
        float top = t00 * (1.0f - a) + t10 * a;
        float bot = t01 * (1.0f - a) + t11 * a;
        r[k] = top * (1.0f - b) + bot * b;
    }
    return v3(r[0], r[1], r[2]);
}

void tex_array4(const View& V, float u, float v, float layer, float out[4])
{
    int l = (int)floorf(layer + 0.5f);
    l = l < 0 ? 0 : (l >= V.num_tex ? V.num_tex - 1 : l);
    const uint8_t* base = V.tex + (size_t)l * V.tex_w * V.tex_h * 4;
    int w = V.tex_w, h = V.tex_h;
    float xf = u * (float)w - 0.5f, yf = v * (float)h - 0.5f;
    float x0f = floorf(xf), y0f = floorf(yf);
    float a = xf - x0f, b = yf - y0f;
    int x0 = wrapi((int)x0f, w), x1 = wrapi((int)x0f + 1, w), y0 = wrapi((int)y0f, h), y1 = wrapi((int)y0f + 1, h);
    for (int k = 0; k < 4; ++k)
    {
        float t00 = base[((size_t)y0 * w + x0) * 4 + k] / 255.0f, t10 = base[((size_t)y0 * w + x1) * 4 + k] / 255.0f;
        float t01 = base[((size_t)y1 * w + x0) * 4 + k] / 255.0f, t11 = base[((size_t)y1 * w + x1) * 4 + k] / 255.0f;
        float top = t00 * (1.0f - a) + t10 * a;
        float bot = t01 * (1.0f - a) + t11 * a;
        out[k] = top * (1.0f - b) + bot * b;
    }
}

// ------------------------------------------------------------------ shader state
struct Material
{
    v3 albedo;
    float specular;
    v3 emission;
    float anisotropic, metallic, roughness, subsurface, specularTint;
    float sheen, sheenTint, clearcoat, clearcoatRoughness;
    float specTrans, ior, atDistance;
    v3 extinction;
    float texIDs[4];
};

struct State
{
    int depth = 0;
    float eta = 0.f;
    float hitDist = 0.f;
    v3 fhp, normal, ffnormal, tangent, bitangent;
    bool isEmitter = false;
    v2 texCoord;
    v3 bary;
    int triPacked = 0;   // triID = vertIndices[triPacked]
    int inst = -1;       // `transform` = transforms[inst]
    int matID = 0;
    Material mat{};
    v3 tempTex;          // tempTexCoords
};

struct Shader
{
    const Prepared& P;
    const Options& O;
    // uniforms
    int maxDepth;
    bool RR;
    int RR_DEPTH;
    bool ENVMAP, CONSTANT_BG;
    v3 bgColor;
    float hdrMultiplier, hdrResolution;
    uint32_t seed[4];
    Counters& c;
    uint64_t lightClamps = 0;

    float rand()
    {
        uint32_t v[4] = {seed[0], seed[1], seed[2], seed[3]};
        for (int k = 0; k < 4; ++k) v[k] = v[k] * 1664525u + 1013904223u;
        v[0] += v[1] * v[3]; v[1] += v[2] * v[0]; v[2] += v[0] * v[1]; v[3] += v[1] * v[2];
        for (int k = 0; k < 4; ++k) v[k] = v[k] ^ (v[k] >> 16u);
        v[0] += v[1] * v[3]; v[1] += v[2] * v[0]; v[2] += v[0] * v[1]; v[3] += v[1] * v[2];
        for (int k = 0; k < 4; ++k) seed[k] = v[k];
        return (float)seed[0] / (float)0xffffffffu;
    }

    // ---- sampling.glsl
    v3 ImportanceSampleGTR1(float rgh, float r1, float r2)
    {
        float a = lfc::fmax_g(0.001f, rgh);
        float a2 = a * a;
        float phi = r1 * TWO_PI;
        float cosTheta = sqrtf((1.0f - lfc::pow_c(a2, 1.0f - r1)) / (1.0f - a2));
        float sinTheta = lfc::clamp_g(sqrtf(1.0f - (cosTheta * cosTheta)), 0.0f, 1.0f);
        float sinPhi = lfc::sin_c(phi);
        float cosPhi = lfc::cos_c(phi);
        return v3(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
    }
    v3 ImportanceSampleGTR2(float rgh, float r1, float r2)
    {
        float a = lfc::fmax_g(0.001f, rgh);
        float phi = r1 * TWO_PI;
        float cosTheta = sqrtf((1.0f - r2) / (1.0f + (a * a - 1.0f) * r2));
        float sinTheta = lfc::clamp_g(sqrtf(1.0f - (cosTheta * cosTheta)), 0.0f, 1.0f);
        float sinPhi = lfc::sin_c(phi);
        float cosPhi = lfc::cos_c(phi);
        return v3(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
    }
    static float SchlickFresnel(float u)
    {
        float m = lfc::clamp_g(1.0f - u, 0.0f, 1.0f);
        float m2 = m * m;
        return m2 * m2 * m;
    }
    static float DielectricFresnel(float cos_theta_i, float eta)
    {
        float sinThetaTSq = eta * eta * (1.0f - cos_theta_i * cos_theta_i);
        if (sinThetaTSq > 1.0f) return 1.0f;
        float cos_theta_t = sqrtf(lfc::fmax_g(1.0f - sinThetaTSq, 0.0f));
        float rs = (eta * cos_theta_t - cos_theta_i) / (eta * cos_theta_t + cos_theta_i);
        float rp = (eta * cos_theta_i - cos_theta_t) / (eta * cos_theta_i + cos_theta_t);
        return 0.5f * (rs * rs + rp * rp);
    }
    static float GTR1(float NDotH, float a)
    {
        if (a >= 1.0f) return (1.0f / PI);
        float a2 = a * a;
        float t = 1.0f + (a2 - 1.0f) * NDotH * NDotH;
        return (a2 - 1.0f) / (PI * lfc::log_c(a2) * t);
    }
    static float GTR2(float NDotH, float a)
    {
        float a2 = a * a;
        float t = 1.0f + (a2 - 1.0f) * NDotH * NDotH;
        return a2 / (PI * t * t);
    }
    static float SmithG_GGX(float NDotV, float alphaG)
    {
        float a = alphaG * alphaG;
        float b = NDotV * NDotV;
        return 1.0f / (NDotV + sqrtf(a + b - a * b));
    }
    static v3 CosineSampleHemisphere(float r1, float r2)
    {
        float r = sqrtf(r1);
        float phi = TWO_PI * r2;
        float x = r * lfc::cos_c(phi);
        float y = r * lfc::sin_c(phi);
        float z = sqrtf(lfc::fmax_g(0.0f, 1.0f - x * x - y * y));
        return v3(x, y, z);
    }
    static v3 UniformSampleSphere(float r1, float r2)
    {
        float z = 1.0f - 2.0f * r1;
        float r = sqrtf(lfc::fmax_g(0.0f, 1.0f - z * z));
        float phi = TWO_PI * r2;
        return v3(r * lfc::cos_c(phi), r * lfc::sin_c(phi), z);
    }
    static float powerHeuristic(float a, float b)
    {
        float t = a * a;
        return t / (b * b + t);
    }

    struct LightSampleRec
    {
        v3 normal, emission, direction;
        float dist = 0.f, pdf = 0.f;
    };
    struct BsdfSampleRec
    {
        v3 L, f;
        float pdf = 0.f;
    };

    void sampleSphereLight(const LightData& light, v3 surfacePos, LightSampleRec& rec)
    {
        float r1 = rand();
        float r2 = rand();
        v3 lightSurfacePos = light.position + UniformSampleSphere(r1, r2) * light.radius;
        rec.direction = lightSurfacePos - surfacePos;
        rec.dist = lfc::length(rec.direction);
        float distSq = rec.dist * rec.dist;
        rec.direction = rec.direction / rec.dist;
        rec.normal = lfc::normalize(lightSurfacePos - light.position);
        rec.emission = light.emission * (float)P.v.num_lights;
        rec.pdf = distSq / (light.area * fabsf(lfc::dot(rec.normal, rec.direction)));
    }
    void sampleRectLight(const LightData& light, v3 surfacePos, LightSampleRec& rec)
    {
        float r1 = rand();
        float r2 = rand();
        v3 lightSurfacePos = light.position + light.u * r1 + light.v * r2;
        rec.direction = lightSurfacePos - surfacePos;
        rec.dist = lfc::length(rec.direction);
        float distSq = rec.dist * rec.dist;
        rec.direction = rec.direction / rec.dist;
        rec.normal = lfc::normalize(lfc::cross(light.u, light.v));
        rec.emission = light.emission * (float)P.v.num_lights;
        rec.pdf = distSq / (light.area * fabsf(lfc::dot(rec.normal, rec.direction)));
    }
    void sampleDistantLight(const LightData& light, v3 surfacePos, LightSampleRec& rec)
    {
        rec.direction = lfc::normalize(light.position - v3(0.0f));
        rec.normal = lfc::normalize(surfacePos - light.position);
        rec.emission = light.emission * (float)P.v.num_lights;
        rec.dist = INF_T;
        rec.pdf = 1.0f;
    }
    void sampleOneLight(const LightData& light, v3 surfacePos, LightSampleRec& rec)
    {
        int type = (int)light.type;
        if (type == 0) sampleRectLight(light, surfacePos, rec);
        else if (type == 1) sampleSphereLight(light, surfacePos, rec);
        else sampleDistantLight(light, surfacePos, rec);
    }

    float EnvPdf(v3 dir)
    {
        const View& V = P.v;
        float theta = lfc::acos_c(lfc::clamp_g(dir.y, -1.0f, 1.0f));
        v2 uv((PI + lfc::atan2_c(dir.z, dir.x)) * (1.0f / TWO_PI), theta * (1.0f / PI));
        float c1[2], c2[2];
        tex_nearest2(V.env_cond, V.env_w, V.env_h, uv.x, uv.y, c1);
        tex_nearest2(V.env_marg, V.env_h, 1, uv.y, 0.0f, c2);
        float pdf = c1[1] * c2[1];
        return (pdf * hdrResolution) / (2.0f * PI * PI * lfc::sin_c(theta));
    }

    void EnvSample(v3& color, v3& dir, float& pdfOut)
    {
        const View& V = P.v;
        float r1 = rand();
        float r2 = rand();
        float m[2], cnd[2];
        tex_nearest2(V.env_marg, V.env_h, 1, r1, 0.0f, m);
        float v = m[0];
        tex_nearest2(V.env_cond, V.env_w, V.env_h, r2, v, cnd);
        float u = cnd[0];
        color = tex_linear3(V.env_rgb, V.env_w, V.env_h, u, v) * hdrMultiplier;
        float a[2], b[2];
        tex_nearest2(V.env_cond, V.env_w, V.env_h, u, v, a);
        tex_nearest2(V.env_marg, V.env_h, 1, v, 0.0f, b);
        float pdf = a[1] * b[1];
        float phi = u * TWO_PI;
        float theta = v * PI;
        if (lfc::sin_c(theta) == 0.0f) pdf = 0.0f;
        dir = v3(-lfc::sin_c(theta) * lfc::cos_c(phi), lfc::cos_c(theta), -lfc::sin_c(theta) * lfc::sin_c(phi));
        pdfOut = (pdf * hdrResolution) / (2.0f * PI * PI * lfc::sin_c(theta));
    }

    v3 EmitterSample(const State& state, float lightPdf, v3 lightEmission, float bsdfPdf)
    {
        if (state.depth == 0) return lightEmission;
        return powerHeuristic(bsdfPdf, lightPdf) * lightEmission;
    }

    // ---- disney.glsl
    v3 EvalDielectricReflection(const State& state, v3 V, v3 N, v3 L, v3 H, float& pdf)
    {
        pdf = 0.0f;
        if (lfc::dot(N, L) <= 0.0f) return v3(0.0f);
        float F = DielectricFresnel(lfc::dot(V, H), state.eta);
        float D = GTR2(lfc::dot(N, H), state.mat.roughness);
        pdf = D * lfc::dot(N, H) * F / (4.0f * fabsf(lfc::dot(V, H)));
        float G = SmithG_GGX(fabsf(lfc::dot(N, L)), state.mat.roughness) * SmithG_GGX(fabsf(lfc::dot(N, V)), state.mat.roughness);
        return state.mat.albedo * F * D * G;
    }
    v3 EvalDielectricRefraction(const State& state, v3 V, v3 N, v3 L, v3 H, float& pdf)
    {
        pdf = 0.0f;
        if (lfc::dot(N, L) >= 0.0f) return v3(0.0f);
        float F = DielectricFresnel(fabsf(lfc::dot(V, H)), state.eta);
        float D = GTR2(lfc::dot(N, H), state.mat.roughness);
        float denomSqrt = lfc::dot(L, H) + lfc::dot(V, H) * state.eta;
        pdf = D * lfc::dot(N, H) * (1.0f - F) * fabsf(lfc::dot(L, H)) / (denomSqrt * denomSqrt);
        float G = SmithG_GGX(fabsf(lfc::dot(N, L)), state.mat.roughness) * SmithG_GGX(fabsf(lfc::dot(N, V)), state.mat.roughness);
        return state.mat.albedo * (1.0f - F) * D * G * fabsf(lfc::dot(V, H)) * fabsf(lfc::dot(L, H)) * 4.0f * state.eta *
               state.eta / (denomSqrt * denomSqrt);
    }
    v3 EvalSpecular(const State& state, v3 Cspec0, v3 V, v3 N, v3 L, v3 H, float& pdf)
    {
        pdf = 0.0f;
        if (lfc::dot(N, L) <= 0.0f) return v3(0.0f);
        float D = GTR2(lfc::dot(N, H), state.mat.roughness);
        pdf = D * lfc::dot(N, H) / (4.0f * lfc::dot(V, H));
        float FH = SchlickFresnel(lfc::dot(L, H));
        v3 F = lfc::mix(Cspec0, v3(1.0f), FH);
        float G = SmithG_GGX(fabsf(lfc::dot(N, L)), state.mat.roughness) * SmithG_GGX(fabsf(lfc::dot(N, V)), state.mat.roughness);
        return F * D * G;
    }
    v3 EvalClearcoat(const State& state, v3 V, v3 N, v3 L, v3 H, float& pdf)
    {
        pdf = 0.0f;
        if (lfc::dot(N, L) <= 0.0f) return v3(0.0f);
        float D = GTR1(lfc::dot(N, H), lfc::mix(0.1f, 0.001f, state.mat.clearcoatRoughness));
        pdf = D * lfc::dot(N, H) / (4.0f * lfc::dot(V, H));
        float FH = SchlickFresnel(lfc::dot(L, H));
        float F = lfc::mix(0.04f, 1.0f, FH);
        float G = SmithG_GGX(lfc::dot(N, L), 0.25f) * SmithG_GGX(lfc::dot(N, V), 0.25f);
        return v3(0.25f * state.mat.clearcoat * F * D * G);
    }
    v3 EvalDiffuse(const State& state, v3 Csheen, v3 V, v3 N, v3 L, v3 H, float& pdf)
    {
        pdf = 0.0f;
        if (lfc::dot(N, L) <= 0.0f) return v3(0.0f);
        pdf = lfc::dot(N, L) * (1.0f / PI);
        float FL = SchlickFresnel(lfc::dot(N, L));
        float FV = SchlickFresnel(lfc::dot(N, V));
        float FH = SchlickFresnel(lfc::dot(L, H));
        float Fss90 = lfc::dot(L, H) * lfc::dot(L, H) * state.mat.roughness;
        float Fss = lfc::mix(1.0f, Fss90, FL) * lfc::mix(1.0f, Fss90, FV);
        float ss = 1.0f * (Fss * (1.0f / (lfc::dot(N, L) + lfc::dot(N, V)) - 0.5f) + 0.5f);
        v3 Fsheen = FH * state.mat.sheen * Csheen;
        return ((1.0f / PI) * (ss + state.mat.subsurface) * state.mat.albedo + Fsheen) * (1.0f - state.mat.metallic);
    }

    v3 DisneySample(State& state, v3 V, v3 N, v3& L, float& pdf)
    {
        pdf = 0.0f;
        v3 f(0.0f);
        float r1 = rand();
        float r2 = rand();
        float diffuseRatio = 0.5f * (1.0f - state.mat.metallic);
        float transWeight = (1.0f - state.mat.metallic) * state.mat.specTrans;
        v3 Cdlin = state.mat.albedo;
        float Cdlum = 0.3f * Cdlin.x + 0.6f * Cdlin.y + 0.1f * Cdlin.z;
        v3 Ctint = Cdlum > 0.0f ? Cdlin / Cdlum : v3(1.0f);
        v3 Cspec0 = lfc::mix(state.mat.specular * 0.08f * lfc::mix(v3(1.0f), Ctint, state.mat.specularTint), Cdlin,
                             state.mat.metallic);
        v3 Csheen = lfc::mix(v3(1.0f), Ctint, state.mat.sheenTint);
        if (rand() < transWeight)
        {
            v3 H = ImportanceSampleGTR2(state.mat.roughness, r1, r2);
            H = state.tangent * H.x + state.bitangent * H.y + N * H.z;
            if (lfc::dot(V, H) < 0.0f) H = -H;
            v3 R = lfc::reflect(-V, H);
            float F = DielectricFresnel(fabsf(lfc::dot(R, H)), state.eta);
            if (rand() < F)
            {
                L = lfc::normalize(R);
                f = EvalDielectricReflection(state, V, N, L, H, pdf);
            }
            else
            {
                L = lfc::normalize(lfc::refract(-V, H, state.eta));
                f = EvalDielectricRefraction(state, V, N, L, H, pdf);
            }
            f = f * transWeight;
            pdf = pdf * transWeight;
        }
        else
        {
            if (rand() < diffuseRatio)
            {
                L = CosineSampleHemisphere(r1, r2);
                L = state.tangent * L.x + state.bitangent * L.y + N * L.z;
                v3 H = lfc::normalize(L + V);
                f = EvalDiffuse(state, Csheen, V, N, L, H, pdf);
                pdf = pdf * diffuseRatio;
            }
            else
            {
                float primarySpecRatio = 1.0f / (1.0f + state.mat.clearcoat);
                if (rand() < primarySpecRatio)
                {
                    v3 H = ImportanceSampleGTR2(state.mat.roughness, r1, r2);
                    H = state.tangent * H.x + state.bitangent * H.y + N * H.z;
                    if (lfc::dot(V, H) < 0.0f) H = -H;
                    L = lfc::normalize(lfc::reflect(-V, H));
                    f = EvalSpecular(state, Cspec0, V, N, L, H, pdf);
                    pdf = pdf * (primarySpecRatio * (1.0f - diffuseRatio));
                }
                else
                {
                    v3 H = ImportanceSampleGTR1(lfc::mix(0.1f, 0.001f, state.mat.clearcoatRoughness), r1, r2);
                    H = state.tangent * H.x + state.bitangent * H.y + N * H.z;
                    if (lfc::dot(V, H) < 0.0f) H = -H;
                    L = lfc::normalize(lfc::reflect(-V, H));
                    f = EvalClearcoat(state, V, N, L, H, pdf);
                    pdf = pdf * ((1.0f - primarySpecRatio) * (1.0f - diffuseRatio));
                }
            }
            f = f * (1.0f - transWeight);
            pdf = pdf * (1.0f - transWeight);
        }
        return f;
    }

    v3 DisneyEval(const State& state, v3 V, v3 N, v3 L, float& pdf)
    {
        v3 H;
        bool refl = lfc::dot(N, L) > 0.0f;
        if (refl) H = lfc::normalize(L + V);
        else H = lfc::normalize(L + V * state.eta);
        if (lfc::dot(V, H) < 0.0f) H = -H;
        float diffuseRatio = 0.5f * (1.0f - state.mat.metallic);
        float primarySpecRatio = 1.0f / (1.0f + state.mat.clearcoat);
        float transWeight = (1.0f - state.mat.metallic) * state.mat.specTrans;
        v3 brdf(0.0f), bsdf(0.0f);
        float brdfPdf = 0.0f, bsdfPdf = 0.0f;
        if (transWeight > 0.0f)
        {
            if (refl) bsdf = EvalDielectricReflection(state, V, N, L, H, bsdfPdf);
            else bsdf = EvalDielectricRefraction(state, V, N, L, H, bsdfPdf);
        }
        float m_pdf;
        if (transWeight < 1.0f)
        {
            v3 Cdlin = state.mat.albedo;
            float Cdlum = 0.3f * Cdlin.x + 0.6f * Cdlin.y + 0.1f * Cdlin.z;
            v3 Ctint = Cdlum > 0.0f ? Cdlin / Cdlum : v3(1.0f);
            v3 Cspec0 = lfc::mix(state.mat.specular * 0.08f * lfc::mix(v3(1.0f), Ctint, state.mat.specularTint), Cdlin,
                                 state.mat.metallic);
            v3 Csheen = lfc::mix(v3(1.0f), Ctint, state.mat.sheenTint);
            brdf = brdf + EvalDiffuse(state, Csheen, V, N, L, H, m_pdf);
            brdfPdf = brdfPdf + m_pdf * diffuseRatio;
            brdf = brdf + EvalSpecular(state, Cspec0, V, N, L, H, m_pdf);
            brdfPdf = brdfPdf + m_pdf * primarySpecRatio * (1.0f - diffuseRatio);
            brdf = brdf + EvalClearcoat(state, V, N, L, H, m_pdf);
            brdfPdf = brdfPdf + m_pdf * (1.0f - primarySpecRatio) * (1.0f - diffuseRatio);
        }
        pdf = lfc::mix(brdfPdf, bsdfPdf, transWeight);
        return lfc::mix(brdf, bsdf, transWeight);
    }

    // ---- pathtrace.glsl
    static void Onb(v3 N, v3& T, v3& B)
    {
        v3 UpVector = fabsf(N.z) < 0.999f ? v3(0, 0, 1) : v3(1, 0, 0);
        T = lfc::normalize(lfc::cross(UpVector, N));
        B = lfc::cross(N, T);
    }

    void GetNormalsAndTexCoord(State& state, v3 rdir)
    {
        const View& V = P.v;
        const int* tri = V.vidx + (size_t)state.triPacked * 3;
        const float* n1 = V.norms + (size_t)tri[0] * 4;
        const float* n2 = V.norms + (size_t)tri[1] * 4;
        const float* n3 = V.norms + (size_t)tri[2] * 4;
        v2 t1(state.tempTex.x, n1[3]), t2(state.tempTex.y, n2[3]), t3(state.tempTex.z, n3[3]);
        state.texCoord = t1 * state.bary.x + t2 * state.bary.y + t3 * state.bary.z;
        v3 normal = lfc::normalize(vec3_of(n1) * state.bary.x + vec3_of(n2) * state.bary.y + vec3_of(n3) * state.bary.z);
        const float* nm = &P.nrm[(size_t)(state.inst < 0 ? 0 : state.inst) * 9];
        normal = lfc::normalize(lfc::mul3(nm, normal));
        state.normal = normal;
        state.ffnormal = lfc::dot(normal, rdir) <= 0.0f ? normal : normal * -1.0f;
        Onb(state.normal, state.tangent, state.bitangent);
    }

    void GetMaterialsAndTextures(State& state, v3 rdir)
    {
        const View& V = P.v;
        const float* p = V.mats + (size_t)state.matID * 28;
        Material mat;
        mat.albedo = v3(p[0], p[1], p[2]);
        mat.specular = p[3];
        mat.emission = v3(p[4], p[5], p[6]);
        mat.anisotropic = p[7];
        mat.metallic = p[8];
        mat.roughness = lfc::fmax_g(p[9], 0.001f);
        mat.subsurface = p[10];
        mat.specularTint = p[11];
        mat.sheen = p[12];
        mat.sheenTint = p[13];
        mat.clearcoat = p[14];
        mat.clearcoatRoughness = p[15];
        mat.specTrans = p[16];
        mat.ior = p[17];
        mat.atDistance = p[18];
        mat.extinction = v3(p[20], p[21], p[22]);
        for (int k = 0; k < 4; ++k) mat.texIDs[k] = p[24 + k];
        v2 texUV = state.texCoord;
        texUV.y = 1.0f - texUV.y;
        float tx[4];
        if ((int)mat.texIDs[0] >= 0)
        {
            tex_array4(V, texUV.x, texUV.y, (float)(int)mat.texIDs[0], tx);
            mat.albedo = mat.albedo * lfc::vpow(v3(tx[0], tx[1], tx[2]), v3(2.2f));
        }
        if ((int)mat.texIDs[1] >= 0)
        {
            tex_array4(V, texUV.x, texUV.y, mat.texIDs[1], tx);
            mat.metallic = tx[0];
            mat.roughness = lfc::fmax_g(tx[1] * tx[1], 0.001f);
        }
        if ((int)mat.texIDs[2] >= 0)
        {
            tex_array4(V, texUV.x, texUV.y, (float)(int)mat.texIDs[2], tx);
            v3 nrm = lfc::normalize(v3(tx[0], tx[1], tx[2]) * 2.0f - 1.0f);
            v3 T, B;
            Onb(state.normal, T, B);
            nrm = T * nrm.x + B * nrm.y + state.normal * nrm.z;
            state.normal = lfc::normalize(nrm);
            state.ffnormal = lfc::dot(state.normal, rdir) <= 0.0f ? state.normal : state.normal * -1.0f;
            Onb(state.normal, state.tangent, state.bitangent);
        }
        if (mat.texIDs[3] >= 0.0f)
        {
            tex_array4(V, texUV.x, texUV.y, mat.texIDs[3], tx);
            mat.emission = lfc::vpow(v3(tx[0], tx[1], tx[2]), v3(2.2f));
        }
        state.mat = mat;
        state.eta = lfc::dot(rdir, state.normal) < 0.0f ? (1.0f / mat.ior) : mat.ior;
    }

    v3 DirectLight(v3 rdir, const State& state)
    {
        v3 Li(0.0f);
        v3 surfacePos = state.fhp + state.normal * EPS;
        BsdfSampleRec bsdf;
        if (ENVMAP && !CONSTANT_BG)
        {
            v3 color, lightDir;
            float lightPdf;
            EnvSample(color, lightDir, lightPdf);
            bool inShadow = AnyHit(P, O, surfacePos, lightDir, INF_T - EPS, c);
            if (!inShadow)
            {
                bsdf.f = DisneyEval(state, -rdir, state.ffnormal, lightDir, bsdf.pdf);
                if (bsdf.pdf > 0.0f)
                {
                    float misWeight = powerHeuristic(lightPdf, bsdf.pdf);
                    if (misWeight > 0.0f)
                        Li = Li + misWeight * bsdf.f * fabsf(lfc::dot(lightDir, state.ffnormal)) * color / lightPdf;
                }
            }
        }
        if (O.lights)
        {
            LightSampleRec rec;
            int n = P.v.num_lights;
            int index = (int)(rand() * (float)n);
            if (index >= n)
            {
                index = n - 1;   // texelFetch past the light texture; defined as the last light
                lightClamps++;
            }
            LightData light = light_fetch(P.v, index);
            sampleOneLight(light, surfacePos, rec);
            if (lfc::dot(rec.direction, rec.normal) < 0.0f)
            {
                bool inShadow = AnyHit(P, O, surfacePos, rec.direction, rec.dist - EPS, c);
                if (!inShadow)
                {
                    bsdf.f = DisneyEval(state, -rdir, state.ffnormal, rec.direction, bsdf.pdf);
                    float weight = 1.0f;
                    if (light.area > 0.0f) weight = powerHeuristic(rec.pdf, bsdf.pdf);
                    if (bsdf.pdf > 0.0f)
                        Li = Li + weight * bsdf.f * fabsf(lfc::dot(state.ffnormal, rec.direction)) * rec.emission / rec.pdf;
                }
            }
        }
        return Li;
    }

    v3 PathTrace(v3 ro, v3 rd, uint64_t& extRays)
    {
        const View& V = P.v;
        v3 radiance(0.0f), throughput(1.0f), absorption(0.0f);
        State state;
        state.inst = -1;
        BsdfSampleRec bsdfSampleRec;
        float lightPdf = 0.f;
        v3 lightEmission;
        for (int depth = 0; depth < maxDepth; depth++)
        {
            state.depth = depth;
            state.isEmitter = false;
            HitRec h;
            h.isEmitter = false;
            h.light = -1;
            h.triPacked = state.triPacked;
            h.inst = state.inst;
            h.matID = state.matID;
            h.bary = state.bary;
            h.fhp = state.fhp;
            h.tempTex = state.tempTex;
            ++extRays;
            float t = ClosestHit(P, O, ro, rd, h, lightPdf, lightEmission, c);
            // the shader's State keeps the fields of the last triangle hit
            state.isEmitter = h.isEmitter;
            state.triPacked = h.triPacked;
            state.inst = h.inst;
            state.matID = h.matID;
            state.bary = h.bary;
            state.fhp = h.fhp;
            state.tempTex = h.tempTex;
            state.hitDist = t;
            if (t == INF_T)
            {
                if (CONSTANT_BG)
                    radiance = radiance + bgColor * throughput;
                else if (ENVMAP)
                {
                    float misWeight = 1.0f;
                    v2 uv((PI + lfc::atan2_c(rd.z, rd.x)) * (1.0f / TWO_PI), lfc::acos_c(rd.y) * (1.0f / PI));
                    if (depth > 0)
                    {
                        float envPdf = EnvPdf(rd);
                        misWeight = powerHeuristic(bsdfSampleRec.pdf, envPdf);
                    }
                    radiance = radiance + misWeight * tex_linear3(V.env_rgb, V.env_w, V.env_h, uv.x, uv.y) * throughput * hdrMultiplier;
                }
                return radiance;
            }
            if (state.inst >= 0)
            {
                GetNormalsAndTexCoord(state, rd);
                GetMaterialsAndTextures(state, rd);
            }
            else
            {
                // depth-0 light hit: the shader's State is all zeros, so the material is 0
                // and the texture coordinate (0, 0)
                state.texCoord = v2(0.f, 0.f);
                state.matID = 0;
                GetMaterialsAndTextures(state, rd);
            }
            if (lfc::dot(state.normal, state.ffnormal) > 0.0f) absorption = v3(0.0f);
            radiance = radiance + state.mat.emission * throughput;
            if (O.lights && state.isEmitter)
            {
                radiance = radiance + EmitterSample(state, lightPdf, lightEmission, bsdfSampleRec.pdf) * throughput;
                break;
            }
            throughput = throughput * lfc::vexp(-absorption * t);
            radiance = radiance + DirectLight(rd, state) * throughput;
            bsdfSampleRec.f = DisneySample(state, -rd, state.ffnormal, bsdfSampleRec.L, bsdfSampleRec.pdf);
            if (lfc::dot(state.ffnormal, bsdfSampleRec.L) < 0.0f)
                absorption = (-lfc::vlog(state.mat.extinction)) / state.mat.atDistance;
            if (bsdfSampleRec.pdf > 0.0f)
                throughput = throughput * (bsdfSampleRec.f * fabsf(lfc::dot(state.ffnormal, bsdfSampleRec.L)) / bsdfSampleRec.pdf);
            else
                break;
            if (RR && depth >= RR_DEPTH)
            {
                float q = lfc::fmin_g(lfc::fmax_g(throughput.x, lfc::fmax_g(throughput.y, throughput.z)) + 0.001f, 0.95f);
                if (rand() > q) break;
                throughput = throughput / q;
            }
            rd = bsdfSampleRec.L;
            ro = state.fhp + rd * EPS;
        }
        return radiance;
    }
};

float map_range(float value, float low1, float high1, float low2, float high2)
{
    return low2 + ((value - low1) * (high2 - low2)) / (high1 - low1);
}

template <class Fn>
void parallel_rows(int n, int threads, Fn fn)
{
    if (threads <= 0)
    {
        unsigned hc = std::thread::hardware_concurrency();
        threads = hc ? (int)hc : 1;
    }
    std::atomic<int> next{0};
    auto work = [&](int tid) {
        for (;;)
        {
            int i = next.fetch_add(1);
            if (i >= n) break;
            fn(i, tid);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work, t);
    work(0);
    for (auto& th : pool) th.join();
}

void prepare(const View& v, Prepared& p)
{
    p.v = v;
    p.inv.resize((size_t)v.num_instances * 16);
    p.nrm.resize((size_t)v.num_instances * 9);
    for (int i = 0; i < v.num_instances; ++i)
    {
        lfc::inverse4(v.xf + (size_t)i * 16, &p.inv[(size_t)i * 16]);
        lfc::normal_matrix(v.xf + (size_t)i * 16, &p.nrm[(size_t)i * 9]);
    }
}
}

extern "C" {

// Scene input: the same fields as lf_scene_view in include/lavaframe_gb300.h.
struct lfo_view
{
    const float* nodes;
    int32_t num_nodes;
    int32_t top_level_index;
    const int32_t* vert_indices;
    int32_t num_tris;
    const float* vertices_uvx;
    const float* normals_uvy;
    int32_t num_vertices;
    const float* materials;
    int32_t num_materials;
    const float* transforms;
    int32_t num_instances;
    const float* lights;
    int32_t num_lights;
    const float* env_rgb;
    const float* env_marginal;
    const float* env_conditional;
    int32_t env_width, env_height;
    const uint8_t* textures;
    int32_t tex_width, tex_height, num_textures;
};

struct lfo_params
{
    int32_t width, height;
    int32_t max_depth;
    int32_t enable_rr, rr_depth;
    int32_t use_env_map;
    int32_t use_constant_bg;
    float bg_color[3];
    float hdr_multiplier;
    float cam_position[3], cam_right[3], cam_up[3], cam_forward[3];
    float cam_fov, cam_focal_dist, cam_aperture;
    uint32_t seed;
    int32_t frame_base;
    int32_t tile_width, tile_height;
};

static View to_view(const lfo_view* s)
{
    View v;
    v.nodes = s->nodes; v.num_nodes = s->num_nodes; v.top = s->top_level_index;
    v.vidx = s->vert_indices; v.num_tris = s->num_tris;
    v.verts = s->vertices_uvx; v.norms = s->normals_uvy; v.num_vertices = s->num_vertices;
    v.mats = s->materials; v.num_materials = s->num_materials;
    v.xf = s->transforms; v.num_instances = s->num_instances;
    v.lights = s->lights; v.num_lights = s->num_lights;
    v.env_rgb = s->env_rgb; v.env_marg = s->env_marginal; v.env_cond = s->env_conditional;
    v.env_w = s->env_width; v.env_h = s->env_height;
    v.tex = s->textures; v.tex_w = s->tex_width; v.tex_h = s->tex_height; v.num_tex = s->num_textures;
    return v;
}

// Closest hit for n rays (8 floats each). hits: 4 x int32 per ray (t bits, instance,
// packed triangle, light). stats (optional): node visits, triangle tests, leaf visits,
// stack overflows. cull_rel < 0 reproduces the shader (no culling). ties (optional): 1 for a
// ray whose closest triangle hit has an equal-distance competitor (a grazing edge or vertex,
// or coincident geometry), where only the visit order decides the answer.
int lfo_trace_closest(const lfo_view* sv, const float* rays, int64_t n, int32_t* hits, int32_t lights, float cull_rel,
                      float cull_abs, int32_t threads, uint64_t* stats, uint8_t* ties)
{
    Prepared P;
    prepare(to_view(sv), P);
    Options O{lights, cull_rel, cull_abs};
    const int chunk = 4096;
    int nchunks = (int)((n + chunk - 1) / chunk);
    std::vector<Counters> cs(threads > 0 ? threads : (std::thread::hardware_concurrency() ? std::thread::hardware_concurrency() : 1));
    parallel_rows(nchunks, (int)cs.size(), [&](int ci, int tid) {
        Counters& c = cs[tid];
        for (int64_t i = (int64_t)ci * chunk; i < n && i < (int64_t)(ci + 1) * chunk; ++i)
        {
            const float* r = rays + i * 8;
            HitRec st{};
            st.isEmitter = false;
            st.light = -1;
            st.triPacked = -1;
            st.inst = -1;
            float lp;
            v3 le;
            float t = ClosestHit(P, O, vec3_of(r), vec3_of(r + 4), st, lp, le, c, r[7]);
            int32_t* o = hits + i * 4;
            std::memcpy(&o[0], &t, 4);
            bool tri = !st.isEmitter && st.triPacked >= 0;
            o[1] = tri ? st.inst : -1;
            o[2] = tri ? st.triPacked : -1;
            o[3] = st.isEmitter ? st.light : -1;
            if (ties) ties[i] = (tri && st.tieT == t) ? 1 : 0;
        }
    });
    if (stats)
    {
        uint64_t s[5] = {0, 0, 0, 0, 0};
        for (auto& c : cs) { s[0] += c.nodes; s[1] += c.tris; s[2] += c.leaves; s[3] += c.overflow; s[4] += c.instances; }
        std::memcpy(stats, s, sizeof s);
    }
    return 0;
}

int lfo_trace_any(const lfo_view* sv, const float* rays, int64_t n, uint8_t* occluded, int32_t lights, float cull_rel,
                  float cull_abs, int32_t threads, uint64_t* stats)
{
    Prepared P;
    prepare(to_view(sv), P);
    Options O{lights, cull_rel, cull_abs};
    const int chunk = 4096;
    int nchunks = (int)((n + chunk - 1) / chunk);
    std::vector<Counters> cs(threads > 0 ? threads : (std::thread::hardware_concurrency() ? std::thread::hardware_concurrency() : 1));
    parallel_rows(nchunks, (int)cs.size(), [&](int ci, int tid) {
        for (int64_t i = (int64_t)ci * chunk; i < n && i < (int64_t)(ci + 1) * chunk; ++i)
        {
            const float* r = rays + i * 8;
            occluded[i] = AnyHit(P, O, vec3_of(r), vec3_of(r + 4), r[7], cs[tid]) ? 1 : 0;
        }
    });
    if (stats)
    {
        uint64_t s[5] = {0, 0, 0, 0, 0};
        for (auto& c : cs) { s[0] += c.nodes; s[1] += c.tris; s[2] += c.leaves; s[3] += c.overflow; s[4] += c.instances; }
        std::memcpy(stats, s, sizeof s);
    }
    return 0;
}

// renderer.glsl main() per pixel and sample, summed in sample order into accum (RGB32F,
// row 0 at the bottom). Pixel rows y with y % row_stride == row_offset are rendered
// (row_stride 1 = full frame). paths (optional): radiance per [sample][pixel] of this call.
// counters (optional): [0] paths, [1] extension rays, [2] node visits, [3] light clamps.
int lfo_render(const lfo_view* sv, const lfo_params* p, int32_t first_sample, int32_t num_samples, float* accum,
               float* paths, int32_t row_stride, int32_t row_offset, int32_t threads, float cull_rel, float cull_abs,
               uint64_t* counters)
{
    Prepared P;
    prepare(to_view(sv), P);
    const View& V = P.v;
    Options O{V.num_lights > 0 ? 1 : 0, cull_rel, cull_abs};
    const int W = p->width, H = p->height;
    const int tileW = p->tile_width > 0 ? p->tile_width : W;
    const int tileH = p->tile_height > 0 ? p->tile_height : H;
    const int ntx = (W + tileW - 1) / tileW, nty = (H + tileH - 1) / tileH;
    const float invNumTilesX = 1.0f / ((float)W / (float)tileW);
    const float invNumTilesY = 1.0f / ((float)H / (float)tileH);
    if (row_stride <= 0) row_stride = 1;
    int nth = threads > 0 ? threads : (std::thread::hardware_concurrency() ? (int)std::thread::hardware_concurrency() : 1);
    std::vector<Counters> cs(nth);
    std::vector<uint64_t> ext(nth, 0), clamps(nth, 0), npaths(nth, 0);
    const bool envData = V.env_rgb && V.env_w > 0;
    parallel_rows(H, nth, [&](int gy, int tid) {
        if (gy % row_stride != row_offset) return;
        int ty = gy / tileH, ly = gy - ty * tileH;
        for (int gx = 0; gx < W; ++gx)
        {
            int tx = gx / tileW, lx = gx - tx * tileW;
            (void)ntx;
            (void)nty;
            float* acc = accum + ((size_t)gy * W + gx) * 3;
            for (int s = 0; s < num_samples; ++s)
            {
                Counters& c = cs[tid];
                Shader sh{P, O, p->max_depth, p->enable_rr != 0, p->rr_depth, p->use_env_map != 0 && envData,
                          p->use_constant_bg != 0, v3(p->bg_color[0], p->bg_color[1], p->bg_color[2]),
                          p->hdr_multiplier, envData ? (float)(V.env_w * V.env_h) : 0.0f, {0, 0, 0, 0}, c};
                // renderer.glsl:27-62
                float TexX = ((float)lx + 0.5f) / (float)tileW;
                float TexY = ((float)ly + 0.5f) / (float)tileH;
                float xoffset = -1.0f + 2.0f * invNumTilesX * (float)tx;
                float yoffset = -1.0f + 2.0f * invNumTilesY * (float)ty;
                float ctx = map_range(TexX, 0.0f, 1.0f, xoffset, xoffset + 2.0f * invNumTilesX);
                float cty = map_range(TexY, 0.0f, 1.0f, yoffset, yoffset + 2.0f * invNumTilesY);
                float fsx = map_range(TexX, 0.0f, 1.0f, invNumTilesX * (float)tx, invNumTilesX * (float)tx + invNumTilesX);
                float fsy = map_range(TexY, 0.0f, 1.0f, invNumTilesY * (float)ty, invNumTilesY * (float)ty + invNumTilesY);
                float px = fsx * (float)W, py = fsy * (float)H;
                int frame = p->frame_base + first_sample + s;
                sh.seed[0] = (uint32_t)px;
                sh.seed[1] = (uint32_t)py;
                sh.seed[2] = (uint32_t)frame;
                sh.seed[3] = (uint32_t)px + (uint32_t)py + p->seed * 0x9E3779B9u;
                float r1 = 2.0f * sh.rand();
                float r2 = 2.0f * sh.rand();
                float jx = r1 < 1.0f ? sqrtf(r1) - 1.0f : 1.0f - sqrtf(2.0f - r1);
                float jy = r2 < 1.0f ? sqrtf(r2) - 1.0f : 1.0f - sqrtf(2.0f - r2);
                jx = jx / ((float)W * 0.5f);
                jy = jy / ((float)H * 0.5f);
                float dx = ctx + jx, dy = cty + jy;
                float scale = lfc::tan_c(p->cam_fov * 0.5f);
                dy = dy * ((float)H / (float)W * scale);
                dx = dx * scale;
                v3 right = vec3_of(p->cam_right), up = vec3_of(p->cam_up), fwd = vec3_of(p->cam_forward);
                v3 rayDir = lfc::normalize(dx * right + dy * up + fwd);
                v3 focalPoint = p->cam_focal_dist * rayDir;
                float cam_r1 = sh.rand() * TWO_PI;
                float cam_r2 = sh.rand() * p->cam_aperture;
                v3 randomAperturePos = (lfc::cos_c(cam_r1) * right + lfc::sin_c(cam_r1) * up) * sqrtf(cam_r2);
                v3 finalRayDir = lfc::normalize(focalPoint - randomAperturePos);
                v3 org = vec3_of(p->cam_position) + randomAperturePos;
                v3 col = sh.PathTrace(org, finalRayDir, ext[tid]);
                clamps[tid] += sh.lightClamps;
                npaths[tid]++;
                acc[0] = acc[0] + col.x;
                acc[1] = acc[1] + col.y;
                acc[2] = acc[2] + col.z;
                if (paths)
                {
                    float* o = paths + (((size_t)s * H + gy) * W + gx) * 3;
                    o[0] = col.x; o[1] = col.y; o[2] = col.z;
                }
            }
        }
    });
    if (counters)
    {
        uint64_t s[4] = {0, 0, 0, 0};
        for (int t = 0; t < nth; ++t) { s[0] += npaths[t]; s[1] += ext[t]; s[2] += cs[t].nodes; s[3] += clamps[t]; }
        std::memcpy(counters, s, sizeof s);
    }
    return 0;
}
}

extern "C" {
// Evaluates one contract function element-wise (known-answer tests of the arithmetic
// contract): 0 sin, 1 cos, 2 tan, 3 atan2(x, y), 4 acos, 5 exp, 6 log, 7 pow(x, y).
int lfo_math(int32_t fn, const float* x, const float* y, int64_t n, float* out)
{
    for (int64_t i = 0; i < n; ++i)
    {
        float a = x[i], b = y ? y[i] : 0.f, r = 0.f;
        switch (fn)
        {
        case 0: r = lfc::sin_c(a); break;
        case 1: r = lfc::cos_c(a); break;
        case 2: r = lfc::tan_c(a); break;
        case 3: r = lfc::atan2_c(a, b); break;
        case 4: r = lfc::acos_c(a); break;
        case 5: r = lfc::exp_c(a); break;
        case 6: r = lfc::log_c(a); break;
        case 7: r = lfc::pow_c(a, b); break;
        default: return 1;
        }
        out[i] = r;
    }
    return 0;
}

// Building blocks of disney.glsl / sampling.glsl / intersection.glsl for known-answer tests:
// 0 DielectricFresnel(x, y = eta), 1 GTR2(x = NdotH, y = a), 2 SmithG_GGX(x = NdotV, y = a),
// 3 GTR1(x = NdotH, y = a), 4 SchlickFresnel(x).
int lfo_bsdf_fn(int32_t fn, const float* x, const float* y, int64_t n, float* out)
{
    for (int64_t i = 0; i < n; ++i)
    {
        const float a = x[i], b = y ? y[i] : 0.f;
        float r = 0.f;
        switch (fn)
        {
        case 0: r = Shader::DielectricFresnel(a, b); break;
        case 1: r = Shader::GTR2(a, b); break;
        case 2: r = Shader::SmithG_GGX(a, b); break;
        case 3: r = Shader::GTR1(a, b); break;
        case 4: r = Shader::SchlickFresnel(a); break;
        default: return 1;
        }
        out[i] = r;
    }
    return 0;
}

// AABBIntersect (intersection.glsl:53-68) of n rays (origin xyz, direction xyz) against one
// box (min xyz, max xyz): the shader's return value per ray.
int lfo_aabb(const float* box6, const float* rays6, int64_t n, float* out)
{
    const v3 mn(box6[0], box6[1], box6[2]), mx(box6[3], box6[4], box6[5]);
    for (int64_t i = 0; i < n; ++i)
    {
        const float* r = rays6 + 6 * i;
        float entry;
        out[i] = AABBIntersect(mn, mx, v3(r[0], r[1], r[2]), v3(r[3], r[4], r[5]), &entry);
    }
    return 0;
}

// n DisneySample draws at a surface with normal +z (material: the 26 floats of the shader's
// unpacked material in declaration order - albedo, specular, emission, anisotropic, metallic,
// roughness, subsurface, specularTint, sheen, sheenTint, clearcoat, clearcoatRoughness,
// specTrans, ior, atDistance, extinction, texture ids (ignored); refraction ratio eta; outgoing
// direction V) with the shader's RNG seeded from `seed`; per draw: L xyz, f xyz, pdf, then
// DisneyEval at the same L: f xyz, pdf (11 floats).
static_assert(sizeof(Material) == 26 * sizeof(float), "unpacked material of 26 floats");
int lfo_disney_samples(const float* mat26, float eta, const float* V3, int32_t n, uint32_t seed, float* out)
{
    Prepared P{};
    Options O{0, -1.f, 0.f};
    Counters c{};
    Shader sh{P, O, 1, false, 0, false, false, v3(0.f), 1.f, 0.f, {seed, seed ^ 0x9E3779B9u, 7u, 11u}, c};
    State st{};
    std::memcpy(&st.mat, mat26, sizeof(Material));
    for (int k = 0; k < 4; ++k) st.mat.texIDs[k] = -1.f;
    st.eta = eta;
    st.normal = st.ffnormal = v3(0.f, 0.f, 1.f);
    st.tangent = v3(1.f, 0.f, 0.f);
    st.bitangent = v3(0.f, 1.f, 0.f);
    const v3 V(V3[0], V3[1], V3[2]);
    for (int i = 0; i < n; ++i)
    {
        v3 L;
        float pdf = 0.f, pdfE = 0.f;
        const v3 f = sh.DisneySample(st, V, st.ffnormal, L, pdf);
        const v3 fe = sh.DisneyEval(st, V, st.ffnormal, L, pdfE);
        float* o = out + 11 * i;
        o[0] = L.x; o[1] = L.y; o[2] = L.z;
        o[3] = f.x; o[4] = f.y; o[5] = f.z;
        o[6] = pdf;
        o[7] = fe.x; o[8] = fe.y; o[9] = fe.z;
        o[10] = pdfE;
    }
    return 0;
}

// PCG4D random sequence of the shader (globals.glsl:116-133) for one pixel/frame.
int lfo_rand_sequence(float px, float py, int32_t frame, uint32_t seed_fold, int32_t n, float* out)
{
    uint32_t v[4] = {(uint32_t)px, (uint32_t)py, (uint32_t)frame, (uint32_t)px + (uint32_t)py + seed_fold * 0x9E3779B9u};
    for (int i = 0; i < n; ++i)
    {
        for (int k = 0; k < 4; ++k) v[k] = v[k] * 1664525u + 1013904223u;
        v[0] += v[1] * v[3]; v[1] += v[2] * v[0]; v[2] += v[0] * v[1]; v[3] += v[1] * v[2];
        for (int k = 0; k < 4; ++k) v[k] = v[k] ^ (v[k] >> 16u);
        v[0] += v[1] * v[3]; v[1] += v[2] * v[0]; v[2] += v[0] * v[1]; v[3] += v[1] * v[2];
        out[i] = (float)v[0] / (float)0xffffffffu;
    }
    return 0;
}
}

// ------------------------------------------------------------------ post-process
// postprocess.glsl:26-171 per output pixel, with TiledRenderer's uniforms
// (TiledRenderer.cpp:540-552): GLSL vec4 arithmetic written per component, texture() as the
// accumulation texture's GL_LINEAR / GL_REPEAT sampling (texel centres at +0.5), and the 8-bit
// framebuffer conversion round(clamp(c) * 255) that GetOutputBuffer reads.
namespace
{
struct PostIn
{
    int32_t tonemap, use_ca, use_ca_distortion, use_vignette, preview;
    float ca_distance, ca_p1, ca_p2, ca_p3, vignette_intensity, vignette_power;
};

int wrap(int i, int n)
{
    int r = i % n;
    return r < 0 ? r + n : r;
}

// vec4 texture(pathTraceTexture, uv) of a W x H RGB (alpha 0) image
void texture4(const float* rgb, int W, int H, float u, float v, float out[4])
{
    float xf = u * (float)W - 0.5f, yf = v * (float)H - 0.5f;
    float fx = std::floor(xf), fy = std::floor(yf);
    float a = xf - fx, b = yf - fy;
    int x0 = wrap((int)fx, W), x1 = wrap((int)fx + 1, W), y0 = wrap((int)fy, H), y1 = wrap((int)fy + 1, H);
    for (int k = 0; k < 3; ++k)
    {
        float t00 = rgb[((size_t)y0 * W + x0) * 3 + k], t10 = rgb[((size_t)y0 * W + x1) * 3 + k];
        float t01 = rgb[((size_t)y1 * W + x0) * 3 + k], t11 = rgb[((size_t)y1 * W + x1) * 3 + k];
        out[k] = (t00 * (1.0f - a) + t10 * a) * (1.0f - b) + (t01 * (1.0f - a) + t11 * a) * b;
    }
    out[3] = 0.0f;
}

float glsl_distance(float ax, float ay, float bx, float by)
{
    float dx = ax - bx, dy = ay - by;
    return std::sqrt(dx * dx + dy * dy);
}
}

extern "C" int lfo_postprocess(const float* accum_rgb, int32_t W, int32_t H, const void* params, int32_t samples,
                               uint8_t* rgb8, float* rgbf)
{
    const PostIn& P = *reinterpret_cast<const PostIn*>(params);
    const float invSampleCounter = 1.0f / (float)samples;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
        {
            const float tu = ((float)x + 0.5f) / (float)W, tv = ((float)y + 0.5f) / (float)H;   // TexCoords
            float color[4], t[4];
            if (!P.preview && P.use_ca)
            {
                // chromaticAberration()
                float offset = P.ca_distance;
                float dist = 0.0f + lfc::pow_c(glsl_distance(tu, tv, P.ca_p3, P.ca_p3), P.ca_p1) * P.ca_p2;
                float s;
                if (P.use_ca_distortion)
                    s = offset * dist;
                else
                {
                    offset = offset * 0.025f;
                    s = offset * P.ca_p2;
                }
                texture4(accum_rgb, W, H, tu + s, tv + s, t);
                color[0] = t[0] * invSampleCounter;
                texture4(accum_rgb, W, H, tu, tv, t);
                color[1] = t[1] * invSampleCounter;
                texture4(accum_rgb, W, H, tu - s, tv - s, t);
                color[2] = t[2] * invSampleCounter;
                color[3] = 0.0f;
            }
            else
            {
                texture4(accum_rgb, W, H, tu, tv, t);
                for (int k = 0; k < 4; ++k) color[k] = t[k] * invSampleCounter;
            }
            const float gamma = 1.0f / 2.2f;
            switch (P.tonemap)
            {
            case 1:
            {
                float luminance = 0.3f * color[0] + 0.6f * color[1] + 0.1f * color[2];
                for (int k = 0; k < 4; ++k) color[k] = lfc::pow_c(color[k] * 1.0f / (1.0f + luminance / 2.0f), gamma);
                break;
            }
            case 2:
                for (int k = 0; k < 4; ++k)
                {
                    float c = color[k];
                    color[k] = lfc::pow_c(lfc::clamp_g((c * (2.51f * c + 0.03f)) / (c * (2.43f * c + 0.59f) + 0.14f), 0.0f, 1.0f),
                                          gamma);
                }
                break;
            case 3:
                for (int k = 0; k < 4; ++k) color[k] = lfc::pow_c(lfc::clamp_g(color[k] / (color[k] + 1.0f), 0.0f, 1.0f), gamma);
                break;
            case 4:
                for (int k = 0; k < 4; ++k)
                {
                    float c = color[k];
                    c = lfc::pow_c((c * (c * (1.2295f * c + 0.3135f) + 1.1935f * 0.4655f) / (c * (1.1935f * c + 0.4655f) + 0.073f)),
                                   1.7f);
                    if (k < 3) c = lfc::pow_c(c, 1.0f / 0.8f);
                    c = c * 0.8f;
                    color[k] = lfc::pow_c(lfc::clamp_g(c, 0.0f, 1.0f), gamma);
                }
                break;
            case 5:
                for (int k = 0; k < 4; ++k)
                {
                    float c = lfc::fmax_g(0.0f, color[k] - 0.004f);
                    color[k] = (c * (6.2f * c + 0.5f)) / (c * (6.2f * c + 1.7f) + 0.06f);
                }
                break;
            case 6:
                for (int k = 0; k < 4; ++k)
                {
                    float c = color[k];
                    float u2 = ((c * (0.15f * c + 0.10f * 0.50f) + 0.20f * 0.02f) / (c * (0.15f * c + 0.50f) + 0.20f * 0.30f)) -
                               0.02f / 0.30f;
                    color[k] = lfc::pow_c(u2, gamma) * 1.75f;
                }
                break;
            default:
                break;
            }
            if (P.use_vignette)
            {
                float d = 1.0f - lfc::pow_c(glsl_distance(tu, tv, 0.5f, 0.5f), P.vignette_power) * P.vignette_intensity;
                for (int k = 0; k < 4; ++k) color[k] = color[k] * d;
            }
            const size_t i = (size_t)y * W + x;
            for (int k = 0; k < 3; ++k)
            {
                if (rgbf) rgbf[i * 3 + k] = color[k];
                if (rgb8) rgb8[i * 3 + k] = (uint8_t)std::nearbyint(lfc::clamp_g(color[k], 0.0f, 1.0f) * 255.0f);
            }
        }
    return 0;
}
