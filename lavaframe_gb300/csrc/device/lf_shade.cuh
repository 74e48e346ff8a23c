// Device shading: camera rays, PCG4D random numbers, Disney BSDF sampling/evaluation,
// light and environment sampling, in the arithmetic of the reference shaders
// (shaders/renderer.glsl, shaders/common/{globals,sampling,disney,pathtrace}.glsl).
// Expressions keep the reference's operand order so that every IEEE operation matches
// (this file is compiled with --fmad=false; transcendentals come from lf_contract.h).
#pragma once

#include "lf_device.cuh"

namespace lfd
{
using lfc::v2;
using lfc::v3;

constexpr float kPI = 3.14159265358979323f;        // globals.glsl:6
constexpr float kTWO_PI = 6.28318530717958648f;    // globals.glsl:7

// ------------------------------------------------------------------ RNG (globals.glsl:116-133)
struct Rng
{
    uint32_t x, y, z, w;
};

__device__ __forceinline__ void pcg4d(Rng& v)
{
    v.x = v.x * 1664525u + 1013904223u;
    v.y = v.y * 1664525u + 1013904223u;
    v.z = v.z * 1664525u + 1013904223u;
    v.w = v.w * 1664525u + 1013904223u;
    v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
    v.x ^= v.x >> 16u; v.y ^= v.y >> 16u; v.z ^= v.z >> 16u; v.w ^= v.w >> 16u;
    v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
}

__device__ __forceinline__ float rnd(Rng& s)
{
    pcg4d(s);
    return __uint2float_rn(s.x) / 4294967296.0f;   // float(0xffffffffu) rounds to 2^32
}

// ------------------------------------------------------------------ scene data for shading
struct DevMaterial
{
    float4 p[7];
};

struct ShadeInstance
{
    float fwd[12];   // forward transform columns 0..3 (xyz)
    float nrm[9];    // transpose(inverse(mat3(M))), column-major
    int material;
    int shadeClass;  // material class for sort-by-material: 0 opaque dielectric, 1 metal, 2 transmissive, 3 textured
    float pad;
};

struct EnvMap
{
    const float* rgb;         // W*H*3
    const float2* marginal;   // H
    const float2* cond;       // W*H
    int w, h;
    float resolution;         // float(w*h)
    float multiplier;
};

struct TexArray
{
    const uint8_t* rgba;      // w*h*4 per layer
    int w, h, layers;
};

struct ShadeScene
{
    DevScene trav;
    const int4* vertIndices;   // per packed triangle (x, y, z, -)
    const float4* vertices;    // xyz + u
    const float4* normals;     // xyz + v
    const DevMaterial* materials;
    const ShadeInstance* inst;
    int numMaterials;
    uint32_t shadeClassMask;   // bit k: some instance's material has shade class k
    EnvMap env;
    TexArray tex;
};

struct Params
{
    int width, height;
    int tileX, tileY, tileW, tileH;
    float invNumTilesX, invNumTilesY;
    int maxDepth;
    int rrEnabled, rrDepth;
    int useEnv;          // ENVMAP define and !CONSTANT_BG (env sampling)
    int envOnMiss;       // ENVMAP define (miss lookup)
    int constantBg;
    int useLights;       // LIGHTS define
    float bg[3];
    float cam_pos[3], cam_right[3], cam_up[3], cam_fwd[3];
    float fov, focalDist, aperture;
    uint32_t seed;
    int frameBase;
    int frameStride;     // frame = frameBase + sample * frameStride + tileOrdinal
    int tileOrdinal;
    float hdrMultiplier;
};

// ------------------------------------------------------------------ texture lookups
__device__ __forceinline__ int wrap_repeat(int i, int n)
{
    int r = i % n;
    return r < 0 ? r + n : r;
}

// Nearest, GL_REPEAT: texel floor(u*W) mod W.
__device__ __forceinline__ float2 nearest2(const float2* t, int w, int h, float u, float v)
{
    int x = wrap_repeat((int)floorf(u * (float)w), w);
    int y = wrap_repeat((int)floorf(v * (float)h), h);
    return t[(size_t)y * w + x];
}

// Bilinear, GL_REPEAT: ((T00(1-a) + T10 a)(1-b) + (T01(1-a) + T11 a) b), texel centres at +0.5.
__device__ __forceinline__ v3 bilinear_rgb(const float* t, int w, int h, float u, float v)
{
    float xf = u * (float)w - 0.5f, yf = v * (float)h - 0.5f;
    float fx0 = floorf(xf), fy0 = floorf(yf);
    float a = xf - fx0, b = yf - fy0;
    int x0 = wrap_repeat((int)fx0, w), x1 = wrap_repeat((int)fx0 + 1, w);
    int y0 = wrap_repeat((int)fy0, h), y1 = wrap_repeat((int)fy0 + 1, h);
    const float* p00 = t + ((size_t)y0 * w + x0) * 3;
    const float* p10 = t + ((size_t)y0 * w + x1) * 3;
    const float* p01 = t + ((size_t)y1 * w + x0) * 3;
    const float* p11 = t + ((size_t)y1 * w + x1) * 3;
    float ia = 1.0f - a, ib = 1.0f - b;
    v3 r;
    float c[3];
    for (int k = 0; k < 3; ++k)
    {
        float top = p00[k] * ia + p10[k] * a;
        float bot = p01[k] * ia + p11[k] * a;
        c[k] = top * ib + bot * b;
    }
    r = v3(c[0], c[1], c[2]);
    return r;
}

// RGBA8 array layer, bilinear + GL_REPEAT, channels as byte/255.
__device__ __forceinline__ float4 tex_array(const TexArray& T, float u, float v, float layer)
{
    int l = (int)floorf(layer + 0.5f);
    l = l < 0 ? 0 : (l >= T.layers ? T.layers - 1 : l);
    const uint8_t* base = T.rgba + (size_t)l * T.w * T.h * 4;
    float xf = u * (float)T.w - 0.5f, yf = v * (float)T.h - 0.5f;
    float fx0 = floorf(xf), fy0 = floorf(yf);
    float a = xf - fx0, b = yf - fy0;
    int x0 = wrap_repeat((int)fx0, T.w), x1 = wrap_repeat((int)fx0 + 1, T.w);
    int y0 = wrap_repeat((int)fy0, T.h), y1 = wrap_repeat((int)fy0 + 1, T.h);
    float ia = 1.0f - a, ib = 1.0f - b;
    float c[4];
    for (int k = 0; k < 4; ++k)
    {
        float t00 = base[((size_t)y0 * T.w + x0) * 4 + k] / 255.0f;
        float t10 = base[((size_t)y0 * T.w + x1) * 4 + k] / 255.0f;
        float t01 = base[((size_t)y1 * T.w + x0) * 4 + k] / 255.0f;
        float t11 = base[((size_t)y1 * T.w + x1) * 4 + k] / 255.0f;
        float top = t00 * ia + t10 * a;
        float bot = t01 * ia + t11 * a;
        c[k] = top * ib + bot * b;
    }
    return make_float4(c[0], c[1], c[2], c[3]);
}

// ------------------------------------------------------------------ sampling.glsl
__device__ __forceinline__ v3 ImportanceSampleGTR1(float rgh, float r1, float r2)
{
    float a = lfc::fmax_g(0.001f, rgh);
    float a2 = a * a;
    float phi = r1 * kTWO_PI;
    float cosTheta = sqrtf((1.0f - lfc::pow_c(a2, 1.0f - r1)) / (1.0f - a2));
    float sinTheta = lfc::clamp_g(sqrtf(1.0f - (cosTheta * cosTheta)), 0.0f, 1.0f);
    float s, c;
    lfc::sincos_c(phi, &s, &c);
    return v3(sinTheta * c, sinTheta * s, cosTheta);
}

__device__ __forceinline__ v3 ImportanceSampleGTR2(float rgh, float r1, float r2)
{
    float a = lfc::fmax_g(0.001f, rgh);
    float phi = r1 * kTWO_PI;
    float cosTheta = sqrtf((1.0f - r2) / (1.0f + (a * a - 1.0f) * r2));
    float sinTheta = lfc::clamp_g(sqrtf(1.0f - (cosTheta * cosTheta)), 0.0f, 1.0f);
    float s, c;
    lfc::sincos_c(phi, &s, &c);
    return v3(sinTheta * c, sinTheta * s, cosTheta);
}

__device__ __forceinline__ float SchlickFresnel(float u)
{
    float m = lfc::clamp_g(1.0f - u, 0.0f, 1.0f);
    float m2 = m * m;
    return m2 * m2 * m;
}

__device__ __forceinline__ float DielectricFresnel(float cos_theta_i, float eta)
{
    float sinThetaTSq = eta * eta * (1.0f - cos_theta_i * cos_theta_i);
    if (sinThetaTSq > 1.0f) return 1.0f;
    float cos_theta_t = sqrtf(lfc::fmax_g(1.0f - sinThetaTSq, 0.0f));
    float rs = (eta * cos_theta_t - cos_theta_i) / (eta * cos_theta_t + cos_theta_i);
    float rp = (eta * cos_theta_i - cos_theta_t) / (eta * cos_theta_i + cos_theta_t);
    return 0.5f * (rs * rs + rp * rp);
}

__device__ __forceinline__ float GTR1(float NDotH, float a)
{
    if (a >= 1.0f) return (1.0f / kPI);
    float a2 = a * a;
    float t = 1.0f + (a2 - 1.0f) * NDotH * NDotH;
    return (a2 - 1.0f) / (kPI * lfc::log_c(a2) * t);
}

__device__ __forceinline__ float GTR2(float NDotH, float a)
{
    float a2 = a * a;
    float t = 1.0f + (a2 - 1.0f) * NDotH * NDotH;
    return a2 / (kPI * t * t);
}

__device__ __forceinline__ float SmithG_GGX(float NDotV, float alphaG)
{
    float a = alphaG * alphaG;
    float b = NDotV * NDotV;
    return 1.0f / (NDotV + sqrtf(a + b - a * b));
}

__device__ __forceinline__ v3 CosineSampleHemisphere(float r1, float r2)
{
    float r = sqrtf(r1);
    float phi = kTWO_PI * r2;
    float s, c;
    lfc::sincos_c(phi, &s, &c);
    float x = r * c, y = r * s;
    float z = sqrtf(lfc::fmax_g(0.0f, 1.0f - x * x - y * y));
    return v3(x, y, z);
}

__device__ __forceinline__ v3 UniformSampleSphere(float r1, float r2)
{
    float z = 1.0f - 2.0f * r1;
    float r = sqrtf(lfc::fmax_g(0.0f, 1.0f - z * z));
    float phi = kTWO_PI * r2;
    float s, c;
    lfc::sincos_c(phi, &s, &c);
    return v3(r * c, r * s, z);
}

__device__ __forceinline__ float powerHeuristic(float a, float b)
{
    float t = a * a;
    return t / (b * b + t);
}

// ------------------------------------------------------------------ surface state
struct Mat
{
    v3 albedo;
    float specular;
    v3 emission;
    float anisotropic;
    float metallic, roughness, subsurface, specularTint;
    float sheen, sheenTint, clearcoat, clearcoatRoughness;
    float specTrans, ior, atDistance;
    v3 extinction;
    float texIDs[4];
};

struct Surf
{
    v3 fhp, normal, ffnormal, tangent, bitangent;
    v2 texCoord;
    float eta;
    Mat mat;
};

// Onb (pathtrace.glsl:7-13)
__device__ __forceinline__ void Onb(v3 N, v3& T, v3& B)
{
    v3 up = fabsf(N.z) < 0.999f ? v3(0.f, 0.f, 1.f) : v3(1.f, 0.f, 0.f);
    T = lfc::normalize(lfc::cross(up, N));
    B = lfc::cross(N, T);
}

__device__ __forceinline__ Mat load_material(const ShadeScene& S, int id)
{
    const DevMaterial& m = S.materials[id];
    float4 p1 = m.p[0], p2 = m.p[1], p3 = m.p[2], p4 = m.p[3], p5 = m.p[4], p6 = m.p[5], p7 = m.p[6];
    Mat r;
    r.albedo = v3(p1.x, p1.y, p1.z);
    r.specular = p1.w;
    r.emission = v3(p2.x, p2.y, p2.z);
    r.anisotropic = p2.w;
    r.metallic = p3.x;
    r.roughness = lfc::fmax_g(p3.y, 0.001f);
    r.subsurface = p3.z;
    r.specularTint = p3.w;
    r.sheen = p4.x;
    r.sheenTint = p4.y;
    r.clearcoat = p4.z;
    r.clearcoatRoughness = p4.w;
    r.specTrans = p5.x;
    r.ior = p5.y;
    r.atDistance = p5.z;
    r.extinction = v3(p6.x, p6.y, p6.z);
    r.texIDs[0] = p7.x; r.texIDs[1] = p7.y; r.texIDs[2] = p7.z; r.texIDs[3] = p7.w;
    return r;
}

__device__ __forceinline__ v3 pow22(v3 c) { return lfc::vpow(c, v3(2.2f)); }

// GetMaterialsAndTextures (pathtrace.glsl:40-123) without the texture maps that only
// change emission; `emissionOnly` serves the stale-state evaluation on light hits.
__device__ __forceinline__ void apply_textures(const ShadeScene& S, Surf& s, v3 rdir)
{
    Mat& mat = s.mat;
    v2 texUV = s.texCoord;
    texUV.y = 1.0f - texUV.y;
    if ((int)mat.texIDs[0] >= 0)
    {
        float4 t = tex_array(S.tex, texUV.x, texUV.y, (float)(int)mat.texIDs[0]);
        mat.albedo = mat.albedo * pow22(v3(t.x, t.y, t.z));
    }
    if ((int)mat.texIDs[1] >= 0)
    {
        float4 t = tex_array(S.tex, texUV.x, texUV.y, mat.texIDs[1]);
        mat.metallic = t.x;
        mat.roughness = lfc::fmax_g(t.y * t.y, 0.001f);
    }
    if ((int)mat.texIDs[2] >= 0)
    {
        float4 t = tex_array(S.tex, texUV.x, texUV.y, (float)(int)mat.texIDs[2]);
        v3 nrm = lfc::normalize(v3(t.x, t.y, t.z) * 2.0f - 1.0f);
        v3 T, B;
        Onb(s.normal, T, B);
        nrm = T * nrm.x + B * nrm.y + s.normal * nrm.z;
        s.normal = lfc::normalize(nrm);
        s.ffnormal = lfc::dot(s.normal, rdir) <= 0.0f ? s.normal : s.normal * -1.0f;
        Onb(s.normal, s.tangent, s.bitangent);
    }
    if (mat.texIDs[3] >= 0.0f)
    {
        float4 t = tex_array(S.tex, texUV.x, texUV.y, mat.texIDs[3]);
        mat.emission = pow22(v3(t.x, t.y, t.z));
    }
}

// Texture maps of a surface, out of line (most scenes have none; the check stays inline).
static __device__ __noinline__ Surf apply_texture_maps(const ShadeScene S, Surf s, v3 rdir)
{
    apply_textures(S, s, rdir);
    return s;
}

__device__ __forceinline__ bool has_texture_maps(const Mat& m)
{
    return (int)m.texIDs[0] >= 0 || (int)m.texIDs[1] >= 0 || (int)m.texIDs[2] >= 0 || m.texIDs[3] >= 0.0f;
}

// Emission of a material evaluated at a texture coordinate (texture map included).
__device__ __forceinline__ v3 material_emission(const ShadeScene& S, int matId, v2 texCoord)
{
    Mat mat = load_material(S, matId);
    if (mat.texIDs[3] >= 0.0f)
    {
        float4 t = tex_array(S.tex, texCoord.x, 1.0f - texCoord.y, mat.texIDs[3]);
        return pow22(v3(t.x, t.y, t.z));
    }
    return mat.emission;
}

// ------------------------------------------------------------------ disney.glsl
struct BsdfCtx
{
    float eta;
    Mat mat;
    v3 T, B;
};

__device__ __forceinline__ v3 EvalDielectricReflection(const BsdfCtx& st, v3 V, v3 N, v3 L, v3 H, float& pdf)
{
    pdf = 0.0f;
    if (lfc::dot(N, L) <= 0.0f) return v3(0.0f);
    float F = DielectricFresnel(lfc::dot(V, H), st.eta);
    float D = GTR2(lfc::dot(N, H), st.mat.roughness);
    pdf = D * lfc::dot(N, H) * F / (4.0f * fabsf(lfc::dot(V, H)));
    float G = SmithG_GGX(fabsf(lfc::dot(N, L)), st.mat.roughness) * SmithG_GGX(fabsf(lfc::dot(N, V)), st.mat.roughness);
    return st.mat.albedo * F * D * G;
}

__device__ __forceinline__ v3 EvalDielectricRefraction(const BsdfCtx& st, v3 V, v3 N, v3 L, v3 H, float& pdf)
{
    pdf = 0.0f;
    if (lfc::dot(N, L) >= 0.0f) return v3(0.0f);
    float F = DielectricFresnel(fabsf(lfc::dot(V, H)), st.eta);
    float D = GTR2(lfc::dot(N, H), st.mat.roughness);
    float denomSqrt = lfc::dot(L, H) + lfc::dot(V, H) * st.eta;
    pdf = D * lfc::dot(N, H) * (1.0f - F) * fabsf(lfc::dot(L, H)) / (denomSqrt * denomSqrt);
    float G = SmithG_GGX(fabsf(lfc::dot(N, L)), st.mat.roughness) * SmithG_GGX(fabsf(lfc::dot(N, V)), st.mat.roughness);
    return st.mat.albedo * (1.0f - F) * D * G * fabsf(lfc::dot(V, H)) * fabsf(lfc::dot(L, H)) * 4.0f * st.eta * st.eta /
           (denomSqrt * denomSqrt);
}

__device__ __forceinline__ v3 EvalSpecular(const BsdfCtx& st, v3 Cspec0, v3 V, v3 N, v3 L, v3 H, float& pdf)
{
    pdf = 0.0f;
    if (lfc::dot(N, L) <= 0.0f) return v3(0.0f);
    float D = GTR2(lfc::dot(N, H), st.mat.roughness);
    pdf = D * lfc::dot(N, H) / (4.0f * lfc::dot(V, H));
    float FH = SchlickFresnel(lfc::dot(L, H));
    v3 F = lfc::mix(Cspec0, v3(1.0f), FH);
    float G = SmithG_GGX(fabsf(lfc::dot(N, L)), st.mat.roughness) * SmithG_GGX(fabsf(lfc::dot(N, V)), st.mat.roughness);
    return F * D * G;
}

__device__ __forceinline__ v3 EvalClearcoat(const BsdfCtx& st, v3 V, v3 N, v3 L, v3 H, float& pdf)
{
    pdf = 0.0f;
    if (lfc::dot(N, L) <= 0.0f) return v3(0.0f);
    float D = GTR1(lfc::dot(N, H), lfc::mix_g(0.1f, 0.001f, st.mat.clearcoatRoughness));
    pdf = D * lfc::dot(N, H) / (4.0f * lfc::dot(V, H));
    float FH = SchlickFresnel(lfc::dot(L, H));
    float F = lfc::mix_g(0.04f, 1.0f, FH);
    float G = SmithG_GGX(lfc::dot(N, L), 0.25f) * SmithG_GGX(lfc::dot(N, V), 0.25f);
    return v3(0.25f * st.mat.clearcoat * F * D * G);
}

__device__ __forceinline__ v3 EvalDiffuse(const BsdfCtx& st, v3 Csheen, v3 V, v3 N, v3 L, v3 H, float& pdf)
{
    pdf = 0.0f;
    if (lfc::dot(N, L) <= 0.0f) return v3(0.0f);
    pdf = lfc::dot(N, L) * (1.0f / kPI);
    float FL = SchlickFresnel(lfc::dot(N, L));
    float FV = SchlickFresnel(lfc::dot(N, V));
    float FH = SchlickFresnel(lfc::dot(L, H));
    float Fss90 = lfc::dot(L, H) * lfc::dot(L, H) * st.mat.roughness;
    float Fss = lfc::mix_g(1.0f, Fss90, FL) * lfc::mix_g(1.0f, Fss90, FV);
    float ss = Fss * (1.0f / (lfc::dot(N, L) + lfc::dot(N, V)) - 0.5f) + 0.5f;
    v3 Fsheen = FH * st.mat.sheen * Csheen;
    return ((1.0f / kPI) * (ss + st.mat.subsurface) * st.mat.albedo + Fsheen) * (1.0f - st.mat.metallic);
}

__device__ __forceinline__ void tints(const Mat& m, v3& Cspec0, v3& Csheen)
{
    v3 Cdlin = m.albedo;
    float Cdlum = 0.3f * Cdlin.x + 0.6f * Cdlin.y + 0.1f * Cdlin.z;
    v3 Ctint = Cdlum > 0.0f ? Cdlin / Cdlum : v3(1.0f);
    Cspec0 = lfc::mix(m.specular * 0.08f * lfc::mix(v3(1.0f), Ctint, m.specularTint), Cdlin, m.metallic);
    Csheen = lfc::mix(v3(1.0f), Ctint, m.sheenTint);
}

// DisneySample (disney.glsl:128-225). Consumes rand() in the reference order.
__device__ __forceinline__ v3 DisneySample(const BsdfCtx& st, Rng& rng, v3 V, v3 N, v3& L, float& pdf)
{
    pdf = 0.0f;
    v3 f(0.0f);
    float r1 = rnd(rng);
    float r2 = rnd(rng);
    float diffuseRatio = 0.5f * (1.0f - st.mat.metallic);
    float transWeight = (1.0f - st.mat.metallic) * st.mat.specTrans;
    v3 Cspec0, Csheen;
    tints(st.mat, Cspec0, Csheen);

    if (rnd(rng) < transWeight)
    {
        v3 H = ImportanceSampleGTR2(st.mat.roughness, r1, r2);
        H = st.T * H.x + st.B * H.y + N * H.z;
        if (lfc::dot(V, H) < 0.0f) H = -H;
        v3 R = lfc::reflect(-V, H);
        float F = DielectricFresnel(fabsf(lfc::dot(R, H)), st.eta);
        if (rnd(rng) < F)
        {
            L = lfc::normalize(R);
            f = EvalDielectricReflection(st, V, N, L, H, pdf);
        }
        else
        {
            L = lfc::normalize(lfc::refract(-V, H, st.eta));
            f = EvalDielectricRefraction(st, V, N, L, H, pdf);
        }
        f = f * transWeight;
        pdf = pdf * transWeight;
    }
    else
    {
        if (rnd(rng) < diffuseRatio)
        {
            L = CosineSampleHemisphere(r1, r2);
            L = st.T * L.x + st.B * L.y + N * L.z;
            v3 H = lfc::normalize(L + V);
            f = EvalDiffuse(st, Csheen, V, N, L, H, pdf);
            pdf = pdf * diffuseRatio;
        }
        else
        {
            float primarySpecRatio = 1.0f / (1.0f + st.mat.clearcoat);
            if (rnd(rng) < primarySpecRatio)
            {
                v3 H = ImportanceSampleGTR2(st.mat.roughness, r1, r2);
                H = st.T * H.x + st.B * H.y + N * H.z;
                if (lfc::dot(V, H) < 0.0f) H = -H;
                L = lfc::normalize(lfc::reflect(-V, H));
                f = EvalSpecular(st, Cspec0, V, N, L, H, pdf);
                pdf = pdf * (primarySpecRatio * (1.0f - diffuseRatio));
            }
            else
            {
                v3 H = ImportanceSampleGTR1(lfc::mix_g(0.1f, 0.001f, st.mat.clearcoatRoughness), r1, r2);
                H = st.T * H.x + st.B * H.y + N * H.z;
                if (lfc::dot(V, H) < 0.0f) H = -H;
                L = lfc::normalize(lfc::reflect(-V, H));
                f = EvalClearcoat(st, V, N, L, H, pdf);
                pdf = pdf * ((1.0f - primarySpecRatio) * (1.0f - diffuseRatio));
            }
        }
        f = f * (1.0f - transWeight);
        pdf = pdf * (1.0f - transWeight);
    }
    return f;
}

// DisneyEval (disney.glsl:228-291).
__device__ __forceinline__ v3 DisneyEval(const BsdfCtx& st, v3 V, v3 N, v3 L, float& pdf)
{
    v3 H;
    bool refl = lfc::dot(N, L) > 0.0f;
    if (refl) H = lfc::normalize(L + V);
    else H = lfc::normalize(L + V * st.eta);
    if (lfc::dot(V, H) < 0.0f) H = -H;

    float diffuseRatio = 0.5f * (1.0f - st.mat.metallic);
    float primarySpecRatio = 1.0f / (1.0f + st.mat.clearcoat);
    float transWeight = (1.0f - st.mat.metallic) * st.mat.specTrans;

    v3 brdf(0.0f), bsdf(0.0f);
    float brdfPdf = 0.0f, bsdfPdf = 0.0f;
    if (transWeight > 0.0f)
    {
        if (refl) bsdf = EvalDielectricReflection(st, V, N, L, H, bsdfPdf);
        else bsdf = EvalDielectricRefraction(st, V, N, L, H, bsdfPdf);
    }
    float m_pdf;
    if (transWeight < 1.0f)
    {
        v3 Cspec0, Csheen;
        tints(st.mat, Cspec0, Csheen);
        brdf = brdf + EvalDiffuse(st, Csheen, V, N, L, H, m_pdf);
        brdfPdf = brdfPdf + m_pdf * diffuseRatio;
        brdf = brdf + EvalSpecular(st, Cspec0, V, N, L, H, m_pdf);
        brdfPdf = brdfPdf + m_pdf * primarySpecRatio * (1.0f - diffuseRatio);
        brdf = brdf + EvalClearcoat(st, V, N, L, H, m_pdf);
        brdfPdf = brdfPdf + m_pdf * (1.0f - primarySpecRatio) * (1.0f - diffuseRatio);
    }
    pdf = lfc::mix_g(brdfPdf, bsdfPdf, transWeight);
    return lfc::mix(brdf, bsdf, transWeight);
}

// ------------------------------------------------------------------ environment
// EnvSample (sampling.glsl:246-265); returns direction and pdf, colour through `color`.
__device__ __forceinline__ float4 EnvSample(const EnvMap& E, Rng& rng, v3& color)
{
    float r1 = rnd(rng);
    float r2 = rnd(rng);
    float v = nearest2(E.marginal, E.h, 1, r1, 0.0f).x;
    float u = nearest2(E.cond, E.w, E.h, r2, v).x;
    color = bilinear_rgb(E.rgb, E.w, E.h, u, v) * E.multiplier;
    float pdf = nearest2(E.cond, E.w, E.h, u, v).y * nearest2(E.marginal, E.h, 1, v, 0.0f).y;
    float phi = u * kTWO_PI;
    float theta = v * kPI;
    float st, ct, sp, cp;
    lfc::sincos_c(theta, &st, &ct);
    lfc::sincos_c(phi, &sp, &cp);
    if (st == 0.0f) pdf = 0.0f;
    return make_float4(-st * cp, ct, -st * sp, (pdf * E.resolution) / (2.0f * kPI * kPI * st));
}

// EnvPdf (sampling.glsl:236-243)
__device__ __forceinline__ float EnvPdf(const EnvMap& E, v3 dir)
{
    float theta = lfc::acos_c(lfc::clamp_g(dir.y, -1.0f, 1.0f));
    float ux = (kPI + lfc::atan2_c(dir.z, dir.x)) * (1.0f / kTWO_PI);
    float uy = theta * (1.0f / kPI);
    float pdf = nearest2(E.cond, E.w, E.h, ux, uy).y * nearest2(E.marginal, E.h, 1, uy, 0.0f).y;
    return (pdf * E.resolution) / (2.0f * kPI * kPI * lfc::sin_c(theta));
}

// Miss contribution before the throughput product (pathtrace.glsl:223-244).
__device__ __forceinline__ v3 env_lookup(const EnvMap& E, v3 dir);

// The environment term of a miss, mis * colour (out of line: misses are a minority of hits).
static __device__ __noinline__ v3 env_miss_term(const EnvMap E, v3 d, int depth, float bsdfPdf);
__device__ __forceinline__ v3 env_lookup(const EnvMap& E, v3 dir)
{
    float ux = (kPI + lfc::atan2_c(dir.z, dir.x)) * (1.0f / kTWO_PI);
    float uy = lfc::acos_c(dir.y) * (1.0f / kPI);
    return bilinear_rgb(E.rgb, E.w, E.h, ux, uy);
}
}

namespace lfd
{
static __device__ __noinline__ v3 env_miss_term(const EnvMap E, v3 d, int depth, float bsdfPdf)
{
    float mis = 1.0f;
    v3 col = env_lookup(E, d);
    if (depth > 0)
    {
        float lightPdf = EnvPdf(E, d);
        mis = powerHeuristic(bsdfPdf, lightPdf);
    }
    return mis * col;
}
}
